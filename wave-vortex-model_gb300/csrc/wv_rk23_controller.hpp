// Step-size controller of the adaptive Bogacki-Shampine RK23 integrator
// (WVAdaptiveRK23, PortableRuntime/src/WVRungeKutta.cpp:554-983; controller
// "matlab-ode23-v1", the step-size rules of MATLAB's ode23).  Plain C++ with
// no CUDA: the stage arithmetic, the right-hand side and the error norm are
// supplied by a backend, so the same controller drives the device integrator
// and can be exercised on the host against the reference's known answers.
//
// Backend interface (each returns WV_SUCCESS or a WV_* code; `message()`
// describes the last failure):
//   int rhs(int slot, bool fromStage, double t);   k[slot] = f(t, base or stage)
//   int affine(int slot, double scale);            stage = base + scale * k[slot]
//   int candidate(double s1, double s2, double s3);
//                                                  stage = ((base + s1 k1) + s2 k2) + s3 k3
//   int error(double h, double relTol, double* e); max over coefficients of
//        |h (b1 k1 + b2 k2 + b3 k3 - k4/8)| / max(absTol, relTol max(|base|, |stage|)),
//        +inf when any ratio is not finite
//   int accept();                                  base = stage
//   void swap_first_last();                        k1 <-> k4 (first same as last)
//   int dense(double h, const double w[4]);        out = stage + sum_i (h w_i) k_i
//   std::string message();
#pragma once

#include "wvgpu.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace wvgpu {

// Time tolerance of interval ends (WVRungeKutta.cpp:21-24).
inline double rk23_time_tolerance(double a, double b) {
    return 8.0 * std::numeric_limits<double>::epsilon() * std::max({1.0, std::abs(a), std::abs(b)});
}

// Validates the options as WVAdaptiveRK23::ensureWorkspace does (WVRungeKutta.cpp:578-588).
inline bool rk23_options_valid(const wv_rk23_options& o) {
    return o.relative_tolerance > 0.0 && o.absolute_tolerance_scale > 0.0 && o.safety_factor > 0.0 &&
           o.safety_factor <= 1.0 && o.rejection_floor_factor > 0.0 && o.rejection_floor_factor < 1.0 &&
           o.maximum_step_factor >= 1.0 && o.maximum_step_factor >= o.rejection_floor_factor &&
           o.maximum_step_size > 0.0;
}

template <class Backend>
class Rk23Controller {
public:
    Rk23Controller(Backend& backend, const wv_rk23_options& options) : b_(backend), o_(options) {}

    const wv_rk23_metrics& metrics() const { return m_; }
    wv_rk23_metrics& metrics() { return m_; }
    const std::vector<wv_rk23_step_diagnostic>& diagnostics() const { return diag_; }
    const std::string& message() const { return msg_; }
    double next_step_size() const { return next_; }
    bool has_accepted_step() const { return hasAccepted_; }
    double accepted_initial_time() const { return hasAccepted_ ? t0Acc_ : 0.0; }
    double accepted_final_time() const { return hasAccepted_ ? t1Acc_ : 0.0; }

    // prepareStateAfterRestart (WVRungeKutta.cpp:645-657).  The constant-
    // stratification system's state constraints only restore forcing
    // amplitudes; the advection and damping schedules have none.
    void restart() {
        hasAccepted_ = false;
        fsal_ = false;
        next_ = 0.0;
        diag_.clear();
    }

    // WVAdaptiveRK23::step (WVRungeKutta.cpp:660-890): one accepted step from t,
    // retrying with smaller steps after rejections; t advances by the accepted step.
    int step(double& t, double proposed) {
        if (stepping_) return fail(WV_REENTRANT_EXECUTION, "RK23 stepping is not reentrant.");
        if (!(proposed > 0.0) || !std::isfinite(proposed))
            return fail(WV_INVALID_CONFIGURATION, "RK23 step size must be finite and positive.");
        if (!rk23_options_valid(o_)) return fail(WV_INVALID_CONFIGURATION, "Adaptive integration tolerances must be positive.");
        stepping_ = true;
        struct Reset {
            bool& v;
            ~Reset() { v = false; }
        } reset{stepping_};
        hasAccepted_ = false;
        const double t0 = t;
        double h = std::min(proposed, o_.maximum_step_size);
        bool haveFirst = false, reused = false;
        if (fsal_) {
            b_.swap_first_last();
            haveFirst = true;
            reused = true;
            fsal_ = false;
            ++m_.fsal_reuses;
        }
        uint64_t rejected = 0, evaluations = 0;
        for (;;) {
            if (!std::isfinite(h) || !(t0 + h > t0)) {
                fsal_ = false;
                return fail(WV_NUMERICAL_FAILURE, "RK23 cannot advance time with the proposed step.");
            }
            int rc;
            if (!haveFirst) {
                if ((rc = b_.rhs(0, false, t0))) return stage_fail(rc);
                ++m_.rhs_evaluations;
                ++evaluations;
                haveFirst = true;
            }
            if ((rc = b_.affine(0, 0.5 * h))) return stage_fail(rc);
            if ((rc = b_.rhs(1, true, t0 + 0.5 * h))) return stage_fail(rc);
            ++m_.rhs_evaluations;
            ++evaluations;
            if ((rc = b_.affine(1, 0.75 * h))) return stage_fail(rc);
            if ((rc = b_.rhs(2, true, t0 + 0.75 * h))) return stage_fail(rc);
            ++m_.rhs_evaluations;
            ++evaluations;
            if ((rc = b_.candidate(h * (2.0 / 9.0), h * (1.0 / 3.0), h * (4.0 / 9.0)))) return stage_fail(rc);
            if ((rc = b_.rhs(3, true, t0 + h))) return stage_fail(rc);
            ++m_.rhs_evaluations;
            ++evaluations;
            double error = 0.0;
            if ((rc = b_.error(h, o_.relative_tolerance, &error))) return stage_fail(rc);
            const bool accepted = std::isfinite(error) && error <= 1.0;
            double factor = 1.0;
            if (accepted) {
                if (rejected == 0) {
                    const double temp = 1.25 * std::cbrt(error);
                    factor = temp > 0.2 ? 1.0 / temp : o_.maximum_step_factor;
                }
            } else if (rejected == 0) {
                factor = std::max(o_.rejection_floor_factor, o_.safety_factor * std::pow(error, -1.0 / 3.0));
            } else {
                factor = o_.rejection_floor_factor;
            }
            next_ = std::min(o_.maximum_step_size, h * factor);
            m_.last_proposed_step_size = proposed;
            m_.normalized_error = error;
            m_.next_step_size = next_;
            if (accepted) {
                if ((rc = b_.accept())) return stage_fail(rc);
                t = t0 + h;
                t0Acc_ = t0;
                t1Acc_ = t;
                ++m_.accepted_steps;
                m_.last_accepted_step_size = h;
                fsal_ = true;  // no state constraint modified the candidate
                hasAccepted_ = true;
                if (diag_.size() < o_.maximum_recorded_step_diagnostics)
                    diag_.push_back({t0, h, error, next_, rejected, evaluations, static_cast<uint8_t>(reused ? 1 : 0)});
                return WV_SUCCESS;
            }
            ++rejected;
            ++m_.rejected_steps;
            ++m_.rejected_initial_derivative_reuses;
            h = next_;
            if (!(h > 0.0) || t0 + h == t0) return fail(WV_NUMERICAL_FAILURE, "RK23 step size underflowed after rejection.");
        }
    }

    // WVAdaptiveRK23::advanceToTime (WVRungeKutta.cpp:892-912).
    int advance_to_time(double& t, double finalTime, double h) {
        if (finalTime < t || !std::isfinite(finalTime))
            return fail(WV_INVALID_CONFIGURATION, "RK23 cannot advance backward or to a nonfinite time.");
        while (t < finalTime) {
            const double remaining = finalTime - t;
            if (remaining <= rk23_time_tolerance(t, finalTime)) break;
            const int rc = step(t, std::min(h, remaining));
            if (rc) return rc;
            h = next_;
        }
        t = finalTime;
        return WV_SUCCESS;
    }

    // WVAdaptiveRK23::evaluateDenseOutput (WVRungeKutta.cpp:914-981): the cubic
    // Hermite interpolant of the last accepted step.
    int dense_output(double time) {
        if (!hasAccepted_) return fail(WV_UNSUPPORTED_OPERATION, "RK23 dense output is unavailable.");
        const double h = t1Acc_ - t0Acc_;
        const double tol = rk23_time_tolerance(t0Acc_, t1Acc_);
        if (time < t0Acc_ - tol || time > t1Acc_ + tol)
            return fail(WV_INVALID_CONFIGURATION, "Dense-output time is outside the accepted interval.");
        double theta = h == 0 ? 0 : (time - t0Acc_) / h;
        if (std::abs(time - t0Acc_) <= tol) theta = 0.0;
        if (std::abs(time - t1Acc_) <= tol) theta = 1.0;
        theta = std::max(0.0, std::min(1.0, theta));
        const double t2 = theta * theta, t3 = t2 * theta;
        const double w[4] = {theta - (4.0 / 3.0) * t2 + (5.0 / 9.0) * t3 - 2.0 / 9.0,
                             t2 - (2.0 / 3.0) * t3 - 1.0 / 3.0,
                             (4.0 / 3.0) * t2 - (8.0 / 9.0) * t3 - 4.0 / 9.0,
                             -t2 + t3};
        const int rc = b_.dense(h, w);
        if (rc) return fail(rc, b_.message());
        ++m_.dense_output_evaluations;
        return WV_SUCCESS;
    }

private:
    int fail(int code, const std::string& message) {
        msg_ = message;
        return code;
    }
    int stage_fail(int code) {
        fsal_ = false;
        return fail(code, b_.message());
    }

    Backend& b_;
    wv_rk23_options o_;
    wv_rk23_metrics m_{};
    std::vector<wv_rk23_step_diagnostic> diag_;
    std::string msg_;
    double next_ = 0.0, t0Acc_ = 0.0, t1Acc_ = 0.0;
    bool fsal_ = false, hasAccepted_ = false, stepping_ = false;
};

}  // namespace wvgpu

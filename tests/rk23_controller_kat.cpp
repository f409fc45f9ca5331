// Host-side check of the RK23 step-size controller (wv_rk23_controller.hpp)
// on the reference's own known-answer systems
// (PortableRuntime/tests/TestWVUnifiedIntegration.cpp:100-170,402-478): a
// linear system dy/dt = -y (or dy/dt = 0) with absolute tolerance 1e-10 on
// every element, stepped by a plain host backend.  Prints one JSON object per
// case.  Test infrastructure: built and run by tests/test_rk23_controller.py.
#include "wv_rk23_controller.hpp"

#include <complex>
#include <cstdio>
#include <utility>
#include <vector>

namespace {

using cd = std::complex<double>;

struct LinearBackend {
    std::vector<cd>* base = nullptr;
    std::vector<cd> stage, k[4], interp;
    bool zero = false;
    double atol = 1e-10;

    explicit LinearBackend(size_t n) : stage(n), interp(n) { for (auto& v : k) v.resize(n); }
    int rhs(int slot, bool fromStage, double) {
        const auto& x = fromStage ? stage : *base;
        for (size_t i = 0; i < x.size(); ++i) k[slot][i] = zero ? cd(0.0, 0.0) : cd(-x[i].real(), -x[i].imag());
        return WV_SUCCESS;
    }
    int affine(int slot, double s) {
        for (size_t i = 0; i < stage.size(); ++i)
            stage[i] = cd((*base)[i].real() + s * k[slot][i].real(), (*base)[i].imag() + s * k[slot][i].imag());
        return WV_SUCCESS;
    }
    int candidate(double s1, double s2, double s3) {
        for (size_t i = 0; i < stage.size(); ++i) {
            double re = (*base)[i].real() + s1 * k[0][i].real(), im = (*base)[i].imag() + s1 * k[0][i].imag();
            re = re + s2 * k[1][i].real(); im = im + s2 * k[1][i].imag();
            stage[i] = cd(re + s3 * k[2][i].real(), im + s3 * k[2][i].imag());
        }
        return WV_SUCCESS;
    }
    int error(double h, double relTol, double* e) {
        const double b1 = 2.0 / 9.0 - 7.0 / 24.0, b2 = 1.0 / 3.0 - 0.25, b3 = 4.0 / 9.0 - 1.0 / 3.0;
        double worst = 0.0;
        for (size_t i = 0; i < stage.size(); ++i) {
            const double er = h * (b1 * k[0][i].real() + b2 * k[1][i].real() + b3 * k[2][i].real() - 0.125 * k[3][i].real());
            const double ei = h * (b1 * k[0][i].imag() + b2 * k[1][i].imag() + b3 * k[2][i].imag() - 0.125 * k[3][i].imag());
            const double scale = std::max(atol, relTol * std::max(std::abs((*base)[i]), std::abs(stage[i])));
            const double r = std::hypot(er, ei) / scale;
            if (!std::isfinite(r)) { *e = std::numeric_limits<double>::infinity(); return WV_SUCCESS; }
            worst = std::max(worst, r);
        }
        *e = worst;
        return WV_SUCCESS;
    }
    int accept() { *base = stage; return WV_SUCCESS; }
    void swap_first_last() { std::swap(k[0], k[3]); }
    int dense_out(double h, const double w[4]) {
        for (size_t i = 0; i < stage.size(); ++i) {
            cd v = stage[i];
            for (int d = 0; d < 4; ++d) v = cd(v.real() + h * w[d] * k[d][i].real(), v.imag() + h * w[d] * k[d][i].imag());
            interp[i] = v;
        }
        return WV_SUCCESS;
    }
    int dense(double h, const double w[4]) { return dense_out(h, w); }
    std::string message() const { return "linear backend"; }
};

void report(const char* name, const wvgpu::Rk23Controller<LinearBackend>& c, const std::vector<cd>& y, double t, int rc,
            double dense0re) {
    const auto& m = c.metrics();
    const auto& d = c.diagnostics();
    std::printf("{\"case\": \"%s\", \"rc\": %d, \"last_step\": %.17g, \"t\": %.17g, \"accepted\": %llu, \"rejected\": %llu, \"evaluations\": %llu, "
                "\"fsal_reuses\": %llu, \"diagnostics\": %zu, \"first_step\": %.17g, \"first_fsal\": %d, \"last_fsal\": %d, "
                "\"max_diag_error\": %.17g, \"y0\": [%.17g, %.17g], \"dense0\": %.17g, \"next\": %.17g}\n",
                name, rc, c.accepted_final_time() - c.accepted_initial_time(), t, (unsigned long long)m.accepted_steps, (unsigned long long)m.rejected_steps,
                (unsigned long long)m.rhs_evaluations, (unsigned long long)m.fsal_reuses, d.size(),
                d.empty() ? 0.0 : d.front().accepted_step_size, d.empty() ? -1 : d.front().reused_fsal_derivative,
                d.empty() ? -1 : d.back().reused_fsal_derivative,
                [&] { double e = 0; for (const auto& x : d) e = std::max(e, x.normalized_error); return e; }(),
                y[0].real(), y[0].imag(), dense0re, c.next_step_size());
}

}  // namespace

int main() {
    wv_rk23_options o{1e-3, 1e-6, 0.8, 0.5, 5.0, std::numeric_limits<double>::infinity(), 512};
    {
        // MATLAB ode23 parity: one coefficient per component, (1, 0.5), rtol 1e-8,
        // maximum step 0.5, advanceToTime(1, 0.5)
        std::vector<cd> y(3, cd(1.0, 0.5));
        LinearBackend b(3);
        b.base = &y;
        wv_rk23_options p = o;
        p.relative_tolerance = 1e-8;
        p.absolute_tolerance_scale = 1e-10;
        p.maximum_step_size = 0.5;
        wvgpu::Rk23Controller<LinearBackend> c(b, p);
        double t = 0.0;
        const int rc = c.advance_to_time(t, 1.0, 0.5);
        report("ode23_parity", c, y, t, rc, 0.0);
    }
    {
        // zero derivative on a 2x3 layout, maximum step 0.1: 10 steps, 31 evaluations
        std::vector<cd> y(18, cd(0.0, 0.0));
        LinearBackend b(18);
        b.base = &y;
        b.zero = true;
        wv_rk23_options p = o;
        p.maximum_step_size = 0.1;
        wvgpu::Rk23Controller<LinearBackend> c(b, p);
        double t = 0.0;
        const int rc = c.advance_to_time(t, 1.0, 0.5);
        report("zero_derivative", c, y, t, rc, 0.0);
    }
    {
        // one step from 0.5 with rtol 1e-8, maximum factor 2 (the system's
        // tolerance policy keeps 1e-10 whatever the scale;
        // TestWVUnifiedIntegration.cpp:366-390): rejections, no growth after
        // a rejection, dense output at the midpoint ~ exp(-t)
        std::vector<cd> y(3, cd(1.0, 0.0));
        LinearBackend b(3);
        b.base = &y;
        wv_rk23_options p = o;
        p.relative_tolerance = 1e-8;
        p.absolute_tolerance_scale = 1.0;
        p.maximum_step_factor = 2.0;
        wvgpu::Rk23Controller<LinearBackend> c(b, p);
        double t = 0.0;
        const int rc = c.step(t, 0.5);
        const double mid = 0.5 * (c.accepted_initial_time() + c.accepted_final_time());
        const int rd = c.dense_output(mid);
        report("single_step", c, y, t, rc ? rc : rd, b.interp[0].real() - std::exp(-mid));
    }
    return 0;
}

// Reference-side drop-in (see WVGPUIntegrationSystem.hpp).
#include "WVGPUIntegrationSystem.hpp"

#include "WaveVortexRuntime/WVIntegrationState.hpp"

#include <cstdint>
#include <limits>
#include <new>
#include <string>

namespace wvgpu_adapter {

using wavevortex::WVKernelStatus;
using wavevortex::WVKernelStatusCode;
namespace rt = wavevortex::runtime;

namespace {

const double* cdata(const wavevortex::WVComplexConstView& v) { return reinterpret_cast<const double*>(v.data); }
double* mdata(wavevortex::WVComplexView& v) { return reinterpret_cast<double*>(v.data); }

// Status codes of the C ABI are the reference's WVKernelStatusCode values.
WVKernelStatus fromCode(int rc, const char* message) {
    if (rc == WV_SUCCESS) return WVKernelStatus::ok();
    return {static_cast<WVKernelStatusCode>(rc), message ? message : "GPU kernel call failed."};
}

// Absolute tolerances per coefficient: Ap, Am use the wave tolerances and A0 the
// vortex ones (WVWaveVortexCoefficientErrorPolicy, WVForcingEngine.cpp:79-180).
class CoefficientErrorPolicy final : public rt::WVIntegrationErrorPolicy {
public:
    CoefficientErrorPolicy(std::vector<double> wave, std::vector<double> vortex)
        : wave_(std::move(wave)), vortex_(std::move(vortex)) {}
    std::size_t componentCount() const noexcept override { return 3; }
    std::size_t elementCount(std::size_t component) const noexcept override { return component < 3 ? wave_.size() : 0; }
    double absoluteTolerance(std::size_t component, std::size_t index) const noexcept override {
        if (component > 2 || index >= wave_.size()) return std::numeric_limits<double>::quiet_NaN();
        return component < 2 ? wave_[index] : vortex_[index];
    }
    std::size_t persistentBytes() const noexcept override {
        return sizeof(*this) + (wave_.capacity() + vortex_.capacity()) * sizeof(double);
    }

private:
    std::vector<double> wave_, vortex_;
};

} // namespace

// ---- WVGPUKernelAdapter --------------------------------------------------------------

WVKernelStatus WVGPUKernelAdapter::create(const wavevortex::WVTransformConstantStratificationConfiguration& c,
                                          int precision, std::unique_ptr<WVGPUKernelAdapter>& out) {
    wv_config g{};
    g.contract_version = c.contractVersion;
    g.Nx = c.Nx; g.Ny = c.Ny; g.Nz = c.Nz; g.Nj = c.Nj;
    g.Lx = c.Lx; g.Ly = c.Ly; g.Lz = c.Lz; g.N0 = c.N0; g.rho0 = c.rho0; g.g = c.g;
    g.planetary_radius = c.planetaryRadius; g.rotation_rate = c.rotationRate; g.latitude = c.latitude;
    g.is_hydrostatic = c.isHydrostatic ? 1 : 0;
    g.should_antialias = c.shouldAntialias ? 1 : 0;
    char message[512] = {};
    wv_sizes sizes{};
    int rc = wv_describe(&g, &sizes, message, sizeof(message));
    if (rc != WV_SUCCESS) return fromCode(rc, message);
    wv_handle* h = nullptr;
    rc = wv_create(&g, precision, &h);
    if (rc != WV_SUCCESS) return fromCode(rc, "GPU kernel creation failed.");
    try {
        out.reset(new WVGPUKernelAdapter(h, {static_cast<std::size_t>(sizes.Nj), static_cast<std::size_t>(sizes.Nkl)}));
    } catch (const std::bad_alloc&) {
        wv_destroy(h);
        return {WVKernelStatusCode::allocationFailure, "Unable to allocate the GPU kernel adapter."};
    }
    return WVKernelStatus::ok();
}

WVGPUKernelAdapter::~WVGPUKernelAdapter() { wv_destroy(h_); }

WVKernelStatus WVGPUKernelAdapter::status(int rc) const { return fromCode(rc, wv_last_message(h_)); }

WVKernelStatus WVGPUKernelAdapter::nonlinearFlux(const wavevortex::WVState& s, wavevortex::WVFlux& f) {
    return status(wv_nonlinear_flux(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am),
                                    cdata(s.coefficients.A0), mdata(f.Fp), mdata(f.Fm), mdata(f.F0)));
}

WVKernelStatus WVGPUKernelAdapter::nonlinearFluxWithAdvectionFields(const wavevortex::WVState& s, wavevortex::WVFlux& f,
                                                                    wavevortex::WVRealFieldBundleView& advection) {
    return status(wv_nonlinear_flux_with_advection_fields(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am),
                                                          cdata(s.coefficients.A0), mdata(f.Fp), mdata(f.Fm), mdata(f.F0),
                                                          advection.data));
}

WVKernelStatus WVGPUKernelAdapter::nonlinearFluxUsingAdvectionFields(const wavevortex::WVState& s, wavevortex::WVFlux& f,
                                                                     const wavevortex::WVRealFieldBundleConstView& advection) {
    return status(wv_nonlinear_flux_using_advection_fields(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am),
                                                           cdata(s.coefficients.A0), mdata(f.Fp), mdata(f.Fm), mdata(f.F0),
                                                           advection.data));
}

WVKernelStatus WVGPUKernelAdapter::transformWaveVortexToUVWEta(const wavevortex::WVState& s,
                                                               wavevortex::WVRealFieldBundleView& out) {
    return status(wv_inverse(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am), cdata(s.coefficients.A0),
                             out.data));
}

WVKernelStatus WVGPUKernelAdapter::transformWaveVortexToUVW(const wavevortex::WVState& s,
                                                            wavevortex::WVRealFieldBundleView& out) {
    return status(wv_inverse_uvw(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am),
                                 cdata(s.coefficients.A0), out.data));
}

WVKernelStatus WVGPUKernelAdapter::transformUVWEtaToWaveVortex(const wavevortex::WVRealFieldBundleConstView& in, double t,
                                                               double t0, wavevortex::WVMutableCoefficients& c) {
    return status(wv_forward(h_, in.data, t, t0, mdata(c.Ap), mdata(c.Am), mdata(c.A0)));
}

WVKernelStatus WVGPUKernelAdapter::advectFGridScalar(const wavevortex::WVRealVolumeConstView& scalar,
                                                     const wavevortex::WVRealFieldBundleConstView& advection, bool antialias,
                                                     wavevortex::WVRealVolumeView& rhs) {
    return status(wv_advect_fgrid_scalar(h_, scalar.data, advection.data, antialias ? 1 : 0, rhs.data));
}

WVKernelStatus WVGPUKernelAdapter::setForcing(bool nonlinearAdvection, bool adaptiveDamping) {
    const uint32_t flags = (nonlinearAdvection ? WV_FORCING_NONLINEAR_ADVECTION : 0u) |
                           (adaptiveDamping ? WV_FORCING_ADAPTIVE_DAMPING : 0u);
    return status(wv_set_forcing(h_, flags));
}

WVKernelStatus WVGPUKernelAdapter::evaluateRightHandSide(const wavevortex::WVState& s, wavevortex::WVFlux& f) {
    return status(wv_evaluate_rhs(h_, s.t, s.t0, cdata(s.coefficients.Ap), cdata(s.coefficients.Am),
                                  cdata(s.coefficients.A0), mdata(f.Fp), mdata(f.Fm), mdata(f.F0)));
}

WVKernelStatus WVGPUKernelAdapter::rk4Steps(wavevortex::WVMutableState& s, double dt, int steps) {
    double t = s.t;
    const WVKernelStatus st = status(wv_rk4_steps(h_, mdata(s.coefficients.Ap), mdata(s.coefficients.Am),
                                                  mdata(s.coefficients.A0), &t, s.t0, dt, steps));
    if (st) s.t = t;
    return st;
}

WVKernelStatus WVGPUKernelAdapter::errorTolerances(double scale, std::vector<double>& wave, std::vector<double>& vortex) {
    try {
        wave.assign(shape_.elementCount(), 0.0);
        vortex.assign(shape_.elementCount(), 0.0);
    } catch (const std::bad_alloc&) {
        return {WVKernelStatusCode::allocationFailure, "Adaptive tolerance allocation failed."};
    }
    return status(wv_error_tolerances(h_, scale, wave.data(), vortex.data()));
}

// ---- WVGPUIntegrationSystem ----------------------------------------------------------

WVKernelStatus WVGPUIntegrationSystem::create(const wavevortex::WVTransformConstantStratificationConfiguration& c,
                                              const rt::WVFrozenForcingSchedule& schedule, int precision,
                                              std::unique_ptr<WVGPUIntegrationSystem>& out) {
    bool advection = false, damping = false;
    for (const auto& e : schedule.entries) {
        if (e.typeIdentifier == "WVNonlinearAdvection") advection = true;
        else if (e.typeIdentifier == "WVAdaptiveDamping") damping = true;
        else return {WVKernelStatusCode::unsupportedOperation,
                     "The GPU integration system supports the WVNonlinearAdvection and WVAdaptiveDamping forcings only."};
    }
    if (!advection)
        return {WVKernelStatusCode::unsupportedOperation, "The GPU integration system requires WVNonlinearAdvection."};
    std::unique_ptr<WVGPUIntegrationSystem> s;
    try {
        s.reset(new WVGPUIntegrationSystem());
    } catch (const std::bad_alloc&) {
        return {WVKernelStatusCode::allocationFailure, "Unable to allocate the GPU integration system."};
    }
    auto st = WVGPUKernelAdapter::create(c, precision, s->kernel_);
    if (!st) return st;
    st = s->kernel_->setForcing(true, damping);
    if (!st) return st;
    st = rt::WVIntegrationStateLayout::createCoefficientOnly(s->kernel_->spectralShape(), s->layout_);
    if (!st) return st;
    out = std::move(s);
    return WVKernelStatus::ok();
}

WVKernelStatus WVGPUIntegrationSystem::evaluateRightHandSide(const rt::WVIntegrationState& state,
                                                             rt::WVIntegrationFlux& rightHandSide) {
    auto st = rt::validateIntegrationState(layout_, state);
    if (!st) return st;
    if (rightHandSide.additionalBlockCount != 0)
        return {WVKernelStatusCode::invalidShape, "The GPU integration system carries no additional state blocks."};
    ++evaluations_;
    return kernel_->evaluateRightHandSide(state.waveVortex, rightHandSide.waveVortex);
}

rt::WVStateConstraintResult WVGPUIntegrationSystem::enforceStateConstraints(rt::WVMutableIntegrationState& state) {
    const auto st = rt::validateMutableIntegrationState(layout_, state);
    if (!st) return {st, 0, false};
    // nonlinear advection and adaptive damping have no forcing amplitudes to restore
    return {WVKernelStatus::ok(), 0, true};
}

WVKernelStatus WVGPUIntegrationSystem::createErrorPolicy(double absoluteToleranceScale,
                                                         std::unique_ptr<rt::WVIntegrationErrorPolicy>& policy) const {
    policy.reset();
    std::vector<double> wave, vortex;
    auto st = kernel_->errorTolerances(absoluteToleranceScale, wave, vortex);
    if (!st) return st;
    try {
        policy = std::make_unique<CoefficientErrorPolicy>(std::move(wave), std::move(vortex));
    } catch (const std::bad_alloc&) {
        return {WVKernelStatusCode::allocationFailure, "Integration error-policy allocation failed."};
    }
    return WVKernelStatus::ok();
}

} // namespace wvgpu_adapter

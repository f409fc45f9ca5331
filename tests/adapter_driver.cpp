// Test driver: the reference's own integrators (WVFixedStepRK4 and
// WVAdaptiveRK23, PortableRuntime/src/WVRungeKutta.cpp:335-462,554-983) stepping
// the reference-side drop-in WVGPUIntegrationSystem, whose right-hand side runs
// on the GPU through the C ABI.  Built by tests/test_adapter.py against the
// reference build (oracle/_ref/libwvref.so: the integrators and state-layout
// code) and libwvgpu.so.
#include "WVGPUIntegrationSystem.hpp"

#include "WaveVortexRuntime/WVRungeKutta.hpp"

#include <cstdint>
#include <memory>
#include <string>

using namespace wavevortex;
using namespace wavevortex::runtime;

namespace {

struct Driver {
    std::unique_ptr<wvgpu_adapter::WVGPUIntegrationSystem> system;
    std::string message;
};

WVComplexView view(double* p, WVShape2D s) { return {reinterpret_cast<WVComplex64*>(p), s}; }
WVComplexConstView cview(const double* p, WVShape2D s) { return {reinterpret_cast<const WVComplex64*>(p), s}; }

int fail(Driver* d, const WVKernelStatus& st) {
    if (d) d->message = st.message;
    return static_cast<int>(st.code);
}

WVFrozenForcingEntry entry(const char* type, const char* name, WVForcingStage stage, std::uint8_t priority) {
    WVFrozenForcingEntry e;
    e.typeIdentifier = type;
    e.name = name;
    e.stage = stage;
    e.priority = priority;
    e.sourceGroupPath = "adapter-test";
    e.configuration = {"wave-vortex-forcing-configuration-v1", 1, {}};
    return e;
}

} // namespace

extern "C" {

// sizes = {Nx, Ny, Nz, Nj}; values = {Lx, Ly, Lz, N0, rho0, g, planetaryRadius,
// rotationRate, latitude}; flags = {isHydrostatic, shouldAntialias};
// schedule 0: {nonlinear advection}, 1: + adaptive damping.
int wvad_create(const std::uint64_t* sizes, const double* values, const std::uint8_t* flags, int schedule,
                int precision, void** out) {
    *out = nullptr;
    WVTransformConstantStratificationConfiguration c;
    c.Nx = sizes[0]; c.Ny = sizes[1]; c.Nz = sizes[2]; c.Nj = sizes[3];
    c.Lx = values[0]; c.Ly = values[1]; c.Lz = values[2]; c.N0 = values[3]; c.rho0 = values[4]; c.g = values[5];
    c.planetaryRadius = values[6]; c.rotationRate = values[7]; c.latitude = values[8];
    c.isHydrostatic = flags[0] != 0; c.shouldAntialias = flags[1] != 0;
    WVFrozenForcingSchedule frozen;
    frozen.entries.push_back(entry("WVNonlinearAdvection", "nonlinear", WVForcingStage::spatial, 127));
    if (schedule == 1) frozen.entries.push_back(entry("WVAdaptiveDamping", "adaptive", WVForcingStage::spectral, 100));
    auto d = std::make_unique<Driver>();
    const auto st = wvgpu_adapter::WVGPUIntegrationSystem::create(c, frozen, precision, d->system);
    if (!st) return static_cast<int>(st.code);
    *out = d.release();
    return 0;
}

void wvad_destroy(void* h) { delete static_cast<Driver*>(h); }
const char* wvad_message(void* h) { return h ? static_cast<Driver*>(h)->message.c_str() : ""; }
std::uint64_t wvad_rhs_evaluations(void* h) { return static_cast<Driver*>(h)->system->rightHandSideEvaluations(); }

// WVIntegrationSystem::evaluateRightHandSide of the GPU system.
int wvad_rhs(void* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* Fp, double* Fm,
             double* F0) {
    auto* d = static_cast<Driver*>(h);
    const auto s = d->system->stateLayout().coefficientShape();
    WVIntegrationState state{{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}}, nullptr, 0};
    WVIntegrationFlux flux{{view(Fp, s), view(Fm, s), view(F0, s)}, nullptr, 0};
    const auto st = d->system->evaluateRightHandSide(state, flux);
    return st ? 0 : fail(d, st);
}

// `steps` steps of the reference's WVFixedStepRK4 over the GPU system.
int wvad_rk4(void* h, double* Ap, double* Am, double* A0, double* t, double t0, double dt, int steps) {
    auto* d = static_cast<Driver*>(h);
    const auto s = d->system->stateLayout().coefficientShape();
    WVFixedStepRK4 rk4(*d->system);
    WVMutableIntegrationState state{{*t, t0, {view(Ap, s), view(Am, s), view(A0, s)}}, nullptr, 0};
    for (int i = 0; i < steps; ++i) {
        const auto st = rk4.step(state, dt);
        if (!st) return fail(d, st);
    }
    *t = state.waveVortex.t;
    return 0;
}

// The reference's WVAdaptiveRK23 over the GPU system from *t to finalTime;
// opts = {rtol, atolScale, safety, floor, maxFactor, maxStep};
// counts = {accepted, rejected, rhs evaluations, fsal reuses}; hashes =
// {toleranceHash, three component hashes}.
int wvad_rk23(void* h, const double* opts, double* Ap, double* Am, double* A0, double* t, double t0, double finalTime,
              double initialStep, unsigned long long* counts, double* nextStep, unsigned long long* hashes) {
    auto* d = static_cast<Driver*>(h);
    const auto s = d->system->stateLayout().coefficientShape();
    WVAdaptiveRK23Options o;
    o.relativeTolerance = opts[0];
    o.absoluteToleranceScale = opts[1];
    o.safetyFactor = opts[2];
    o.rejectionFloorFactor = opts[3];
    o.maximumStepFactor = opts[4];
    o.maximumStepSize = opts[5];
    WVAdaptiveRK23 rk(*d->system, o);
    WVMutableIntegrationState state{{*t, t0, {view(Ap, s), view(Am, s), view(A0, s)}}, nullptr, 0};
    auto st = rk.prepareStateAfterRestart(state);
    if (!st) return fail(d, st);
    st = rk.advanceToTime(state, finalTime, initialStep);
    if (!st) return fail(d, st);
    *t = state.waveVortex.t;
    counts[0] = rk.metrics().acceptedStepCount;
    counts[1] = rk.metrics().rejectedStepCount;
    counts[2] = rk.metrics().rightHandSideEvaluationCount;
    counts[3] = rk.metrics().fsalReuseCount;
    *nextStep = rk.nextStepSize();
    hashes[0] = rk.toleranceHash();
    for (int c = 0; c < 3; ++c) hashes[1 + c] = rk.toleranceComponentHashes()[c];
    return 0;
}

} // extern "C"

// Test infrastructure only: a C entry layer over the UNMODIFIED reference
// CompiledKernel + PortableRuntime sources, compiled by oracle/ref_build.sh
// into oracle/_ref/libwvref.so.  It is used to generate golden fixtures and
// to pin the numpy oracle; the shipped GPU path never links or loads it.
//
// Reference interfaces driven here:
//   WVTransformConstantStratificationKernel::create / nonlinearFlux /
//     transformUVWEtaToWaveVortex / transformUVEtaToWaveVortex /
//     transformWaveVortexToUVWEta
//     (CompiledKernel/include/WaveVortexKernel/WVTransformConstantStratificationKernel.hpp:47-110)
//   WVConstantStratificationIntegrationSystem::create / evaluateRightHandSide
//     (PortableRuntime/include/WaveVortexRuntime/WVConstantStratificationIntegrationSystem.hpp:40-66)
//   WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462)
//   WVReferenceFFTEngine, the exact direct DFT/DCT-I/DST-I engine
//     (CompiledKernel/adapters/reference/WVReferenceFFTEngine.cpp:47-107), or
//   wvoracle::OracleFFTEngine (oracle/wv_fft_engine.cpp), an O(N log N)
//     provider of the same contract for grids the direct engine cannot reach

#include "WVReferenceFFTEngine.hpp"
#include "wv_fft_engine.hpp"
#include "WaveVortexKernel/WVTransformConstantStratificationKernel.hpp"
#include "WaveVortexRuntime/WVConstantStratificationIntegrationSystem.hpp"
#include "WaveVortexRuntime/WVExtensionCatalog.hpp"
#include "WaveVortexRuntime/WVForcingContracts.hpp"
#include "WaveVortexRuntime/WVRungeKutta.hpp"

#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

using namespace wavevortex;
using namespace wavevortex::runtime;

namespace {

struct RefHandle {
    std::unique_ptr<WVTransformConstantStratificationKernel> kernel;
    std::unique_ptr<WVConstantStratificationIntegrationSystem> system;
    std::unique_ptr<WVFixedStepRK4> rk4;
    std::string message;
};

WVTransformConstantStratificationConfiguration makeConfiguration(const std::uint64_t* sizes, const double* values, const std::uint8_t* flags) {
    WVTransformConstantStratificationConfiguration c;
    c.Nx = sizes[0]; c.Ny = sizes[1]; c.Nz = sizes[2]; c.Nj = sizes[3];
    c.Lx = values[0]; c.Ly = values[1]; c.Lz = values[2]; c.N0 = values[3];
    c.rho0 = values[4]; c.g = values[5]; c.planetaryRadius = values[6];
    c.rotationRate = values[7]; c.latitude = values[8];
    c.isHydrostatic = flags[0] != 0; c.shouldAntialias = flags[1] != 0;
    return c;
}

WVFrozenForcingEntry forcingEntry(const char* type, const char* name, WVForcingStage stage, std::uint8_t priority) {
    WVFrozenForcingEntry e;
    e.typeIdentifier = type;
    e.name = name;
    e.stage = stage;
    e.priority = priority;
    e.sourceGroupPath = "oracle";
    e.configuration = {"wave-vortex-forcing-configuration-v1", 1, {}};
    return e;
}

int fail(RefHandle* h, const WVKernelStatus& status) {
    if (h) h->message = status.message;
    return static_cast<int>(status.code);
}

WVComplexConstView cview(const double* p, WVShape2D s) { return {reinterpret_cast<const WVComplex64*>(p), s}; }
WVComplexView mview(double* p, WVShape2D s) { return {reinterpret_cast<WVComplex64*>(p), s}; }

struct RefSystem {
    std::unique_ptr<WVConstantStratificationIntegrationSystem> system;
    std::string message;
    std::size_t M = 0;
};

int sys_fail(RefSystem* h, const WVKernelStatus& status) {
    if (h) h->message = status.message;
    return static_cast<int>(status.code);
}

// Views of a packed additional state (blocks back to back, layout order).
std::vector<WVAdditionalStateBlockView> blockViews(const WVConstantStratificationIntegrationSystem& s, double* packed) {
    std::vector<WVAdditionalStateBlockView> v;
    std::size_t off = 0;
    for (const auto& b : s.stateLayout().additionalBlocks()) {
        v.push_back({&b, packed + off, nullptr});
        off += b.elementCount;
    }
    return v;
}

// engine: 0 = the reference's direct DFT engine, 1 = the oracle's O(N log N) engine
std::unique_ptr<WVFFTEngine> makeEngine(int engine) {
    if (engine == 1) return std::make_unique<wvoracle::OracleFFTEngine>();
    return std::make_unique<WVReferenceFFTEngine>();
}

} // namespace

extern "C" {

// Threads the oracle FFT engine uses (WV_ORACLE_FFT_THREADS or every hardware thread).
unsigned wvref_oracle_fft_threads() { return wvoracle::defaultOracleFFTThreads(); }

// schedule: 0 = {nonlinear advection}; 1 = {nonlinear advection, adaptive damping};
// engine as makeEngine.  The kernel and the integration system each own an engine.
int wvref_create_engine(const std::uint64_t* sizes, const double* values, const std::uint8_t* flags, int schedule,
                        int engine, void** out) {
    auto h = std::make_unique<RefHandle>();
    const auto c = makeConfiguration(sizes, values, flags);
    auto status = WVTransformConstantStratificationKernel::create(c, makeEngine(engine), h->kernel);
    if (!status) { *out = nullptr; return static_cast<int>(status.code); }
    WVFrozenForcingSchedule frozen;
    frozen.entries.push_back(forcingEntry("WVNonlinearAdvection", "nonlinear", WVForcingStage::spatial, 127));
    if (schedule == 1) frozen.entries.push_back(forcingEntry("WVAdaptiveDamping", "adaptive", WVForcingStage::spectral, 100));
    std::shared_ptr<const WVExtensionCatalog> catalog;
    status = makeBuiltInExtensionCatalog(catalog);
    if (!status) { *out = nullptr; return static_cast<int>(status.code); }
    status = WVConstantStratificationIntegrationSystem::create(c, frozen, catalog, makeEngine(engine), h->system);
    if (!status) { *out = nullptr; return static_cast<int>(status.code); }
    h->rk4 = std::make_unique<WVFixedStepRK4>(*h->system);
    *out = h.release();
    return 0;
}

int wvref_create(const std::uint64_t* sizes, const double* values, const std::uint8_t* flags, int schedule, void** out) {
    return wvref_create_engine(sizes, values, flags, schedule, 0, out);
}

void wvref_destroy(void* handle) { delete static_cast<RefHandle*>(handle); }

const char* wvref_message(void* handle) { return handle ? static_cast<RefHandle*>(handle)->message.c_str() : ""; }

// out: Nkl, NxHalf, M
void wvref_sizes(void* handle, std::uint64_t* out) {
    const auto& d = static_cast<RefHandle*>(handle)->kernel->descriptor();
    out[0] = d.Nkl();
    out[1] = d.halfSpectrumMappings().NxHalf;
    out[2] = d.spectralShape().elementCount();
}

// Descriptor arrays for ordering / coefficient checks.
// modes: [Nkl] kMode, lMode; omega, fWaveScale, ApmDScaled, A0FromVorticity, A0FromBuoyancy, NA0Field, ApmNProjection [M];
// storage rows + conj flags [Nkl].
void wvref_descriptor(void* handle, std::int64_t* kMode, std::int64_t* lMode, double* omega, double* fWaveScale,
                      double* A0FromVorticity, double* A0FromBuoyancy, double* NA0Field, double* ApmNProjection,
                      double* UApField, double* WApField, std::uint64_t* storageRows, std::uint8_t* conjugated) {
    const auto& d = static_cast<RefHandle*>(handle)->kernel->descriptor();
    const auto& m = d.verticalModes();
    for (std::size_t i = 0; i < d.Nkl(); ++i) {
        kMode[i] = d.fourierModes()[i].kMode;
        lMode[i] = d.fourierModes()[i].lMode;
        storageRows[i] = d.halfSpectrumMappings().storageRowsByWVIndex[i];
        conjugated[i] = d.halfSpectrumMappings().conjugatesStoredValueByWVIndex[i];
    }
    const auto M = d.spectralShape().elementCount();
    std::memcpy(omega, m.omega.data(), M * sizeof(double));
    std::memcpy(fWaveScale, m.fWaveScale.data(), M * sizeof(double));
    std::memcpy(A0FromVorticity, m.A0FromVorticity.data(), M * sizeof(double));
    std::memcpy(A0FromBuoyancy, m.A0FromBuoyancy.data(), M * sizeof(double));
    std::memcpy(NA0Field, m.NA0Field.data(), M * sizeof(double));
    std::memcpy(ApmNProjection, m.ApmNProjection.data(), M * sizeof(double));
    std::memcpy(UApField, m.UApField.data(), M * 2 * sizeof(double));
    std::memcpy(WApField, m.WApField.data(), M * 2 * sizeof(double));
}

// Stage instrumentation of the reference kernel (WVKernelMetrics): enable != 0
// turns it on; out[0..7] = phase, reconstruction, derivative reconstruction,
// product, projection, coefficient assembly, derivative coefficient assembly and
// coefficient projection seconds of the last call.
void wvref_stage_seconds(void* handle, int enable, double* out) {
    auto* h = static_cast<RefHandle*>(handle);
    h->kernel->setStageInstrumentation(enable != 0);
    const auto& m = h->kernel->metrics();
    const double v[8] = {m.phaseSeconds, m.reconstructionSeconds, m.derivativeReconstructionSeconds, m.productSeconds,
                         m.projectionSeconds, m.coefficientAssemblySeconds, m.derivativeCoefficientAssemblySeconds,
                         m.coefficientProjectionSeconds};
    for (int i = 0; i < 8; ++i) out[i] = v[i];
}

int wvref_flux(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
               double* Fp, double* Fm, double* F0) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVFlux flux{mview(Fp, s), mview(Fm, s), mview(F0, s)};
    const auto status = h->kernel->nonlinearFlux(state, flux);
    return status ? 0 : fail(h, status);
}

// Full scheduled right-hand side (nonlinear advection, plus adaptive damping when created with schedule 1).
int wvref_rhs(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
              double* Fp, double* Fm, double* F0) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto s = h->kernel->descriptor().spectralShape();
    WVIntegrationState state{{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}}, nullptr, 0};
    WVIntegrationFlux flux{{mview(Fp, s), mview(Fm, s), mview(F0, s)}, nullptr, 0};
    const auto status = h->system->evaluateRightHandSide(state, flux);
    return status ? 0 : fail(h, status);
}

// nonlinearFluxWithAdvectionFields: flux plus the advecting (u, v, w), [Nx, Ny, Nz, 3].
int wvref_flux_with_advection(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
                              double* Fp, double* Fm, double* F0, double* fields) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVFlux flux{mview(Fp, s), mview(Fm, s), mview(F0, s)};
    WVRealFieldBundleView view{fields, {c.Nx, c.Ny, c.Nz, 3}};
    const auto status = h->kernel->nonlinearFluxWithAdvectionFields(state, flux, view);
    return status ? 0 : fail(h, status);
}

// nonlinearFluxUsingAdvectionFields: flux advected by the given (u, v, w).
int wvref_flux_using_advection(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
                               double* Fp, double* Fm, double* F0, const double* fields) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVFlux flux{mview(Fp, s), mview(Fm, s), mview(F0, s)};
    WVRealFieldBundleConstView view{fields, {c.Nx, c.Ny, c.Nz, 3}};
    const auto status = h->kernel->nonlinearFluxUsingAdvectionFields(state, flux, view);
    return status ? 0 : fail(h, status);
}

// transformWaveVortexToUVW: [Nx, Ny, Nz, 3].
int wvref_inverse_uvw(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0, double* fields) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVRealFieldBundleView view{fields, {c.Nx, c.Ny, c.Nz, 3}};
    const auto status = h->kernel->transformWaveVortexToUVW(state, view);
    return status ? 0 : fail(h, status);
}

// transformStateFieldDerivatives: (d/dx, d/dy, d/dz) of field 0..3 (u, v, w, eta), [Nx, Ny, Nz, 3].
int wvref_field_derivatives(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0, int field,
                            double* out) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVRealFieldBundleView view{out, {c.Nx, c.Ny, c.Nz, 3}};
    const auto status = h->kernel->transformStateFieldDerivatives(state, static_cast<WVDynamicalField>(field), view);
    return status ? 0 : fail(h, status);
}

// advectFGridScalar: -(u d/dx + v d/dy + w d/dz) of an F-grid scalar [Nx, Ny, Nz].
int wvref_advect_scalar(void* handle, const double* scalar, const double* fields, int antialias, double* rhs) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    WVRealVolumeConstView sv{scalar, {c.Nx, c.Ny, c.Nz}};
    WVRealFieldBundleConstView fv{fields, {c.Nx, c.Ny, c.Nz, 3}};
    WVRealVolumeView rv{rhs, {c.Nx, c.Ny, c.Nz}};
    const auto status = h->kernel->advectFGridScalar(sv, fv, antialias != 0, rv);
    return status ? 0 : fail(h, status);
}

// transformToSpatialDomainWith{F,G}AllDerivatives: (value, d/dx, d/dy, d/dz) of the
// F (ffamily = 1) or G field family of (Apm, A0), [Nx, Ny, Nz, 4].
int wvref_family_derivatives(void* handle, int ffamily, const double* Apm, const double* A0, double* fields) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVRealFieldBundleView view{fields, {c.Nx, c.Ny, c.Nz, 4}};
    const auto status = ffamily ? h->kernel->transformToSpatialDomainWithFAllDerivatives(cview(Apm, s), cview(A0, s), view)
                                : h->kernel->transformToSpatialDomainWithGAllDerivatives(cview(Apm, s), cview(A0, s), view);
    return status ? 0 : fail(h, status);
}

int wvref_forward(void* handle, const double* fields, double t, double t0, double* Ap, double* Am, double* A0) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    const std::size_t channels = c.isHydrostatic ? 3 : 4;
    WVRealFieldBundleConstView view{fields, {c.Nx, c.Ny, c.Nz, channels}};
    WVMutableCoefficients out{mview(Ap, s), mview(Am, s), mview(A0, s)};
    const auto status = c.isHydrostatic ? h->kernel->transformUVEtaToWaveVortex(view, t, t0, out)
                                        : h->kernel->transformUVWEtaToWaveVortex(view, t, t0, out);
    return status ? 0 : fail(h, status);
}

int wvref_inverse(void* handle, double t, double t0, const double* Ap, const double* Am, const double* A0, double* fields) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto& c = h->kernel->descriptor().configuration();
    const auto s = h->kernel->descriptor().spectralShape();
    WVState state{t, t0, {cview(Ap, s), cview(Am, s), cview(A0, s)}};
    WVRealFieldBundleView view{fields, {c.Nx, c.Ny, c.Nz, 4}};
    const auto status = h->kernel->transformWaveVortexToUVWEta(state, view);
    return status ? 0 : fail(h, status);
}

// Fixed-step RK4 through the reference integrator; state updated in place, *t advanced.
int wvref_rk4(void* handle, double* Ap, double* Am, double* A0, double* t, double t0, double dt, int steps) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto s = h->kernel->descriptor().spectralShape();
    WVMutableIntegrationState state{{*t, t0, {mview(Ap, s), mview(Am, s), mview(A0, s)}}, nullptr, 0};
    for (int i = 0; i < steps; ++i) {
        const auto status = h->rk4->step(state, dt);
        if (!status) return fail(h, status);
    }
    *t = state.waveVortex.t;
    return 0;
}

// Adaptive RK23 through the reference integrator (WVAdaptiveRK23,
// PortableRuntime/src/WVRungeKutta.cpp:554-983): a fresh integrator with
// options {rtol, atolScale, safety, floor, maxFactor, maxStep} advances the
// state from *t to finalTime.  diag receives up to cap diagnostics as
// {initialTime, step, error, next, rejected, evaluations, reusedFSAL};
// counts = {accepted, rejected, rhs evaluations, fsal reuses}; hashes =
// {toleranceHash, three component hashes}.  When dense is non-null the
// interpolant of the last accepted step is evaluated at denseTime into it
// ([3][M] complex).
int wvref_rk23_advance(void* handle, const double* opts, double* Ap, double* Am, double* A0, double* t, double t0,
                       double finalTime, double initialStep, double* diag, int cap, int* nDiag,
                       unsigned long long* counts, double* nextStep, unsigned long long* hashes, double denseTime,
                       double* dense) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto s = h->kernel->descriptor().spectralShape();
    WVAdaptiveRK23Options o;
    o.relativeTolerance = opts[0];
    o.absoluteToleranceScale = opts[1];
    o.safetyFactor = opts[2];
    o.rejectionFloorFactor = opts[3];
    o.maximumStepFactor = opts[4];
    o.maximumStepSize = opts[5];
    WVAdaptiveRK23 rk(*h->system, o);
    WVMutableIntegrationState state{{*t, t0, {mview(Ap, s), mview(Am, s), mview(A0, s)}}, nullptr, 0};
    auto status = rk.prepareStateAfterRestart(state);
    if (!status) return fail(h, status);
    status = rk.advanceToTime(state, finalTime, initialStep);
    if (!status) return fail(h, status);
    *t = state.waveVortex.t;
    const auto& d = rk.stepDiagnostics();
    *nDiag = static_cast<int>(d.size());
    for (int i = 0; i < cap && i < static_cast<int>(d.size()); ++i) {
        double* r = diag + 7 * i;
        r[0] = d[i].initialTime; r[1] = d[i].acceptedStepSize; r[2] = d[i].normalizedError; r[3] = d[i].nextStepSize;
        r[4] = static_cast<double>(d[i].rejectedAttemptCount); r[5] = static_cast<double>(d[i].rightHandSideEvaluationCount);
        r[6] = d[i].reusedFSALDerivative ? 1.0 : 0.0;
    }
    counts[0] = rk.metrics().acceptedStepCount;
    counts[1] = rk.metrics().rejectedStepCount;
    counts[2] = rk.metrics().rightHandSideEvaluationCount;
    counts[3] = rk.metrics().fsalReuseCount;
    *nextStep = rk.nextStepSize();
    hashes[0] = rk.toleranceHash();
    for (int c = 0; c < 3; ++c) hashes[1 + c] = rk.toleranceComponentHashes()[c];
    if (dense) {
        const std::size_t M = s.elementCount();
        WVMutableIntegrationState out{{0.0, t0, {mview(dense, s), mview(dense + 2 * M, s), mview(dense + 4 * M, s)}}, nullptr, 0};
        status = rk.evaluateDenseOutput(denseTime, out);
        if (!status) return fail(h, status);
    }
    return 0;
}

// ---- integration system with integrated observers -------------------------------
// WVConstantStratificationIntegrationSystem (PortableRuntime/src/
// WVConstantStratificationIntegrationSystem.cpp:112-400) built from an observer
// descriptor: particle groups (x, y[, z] state blocks, linear or spline
// advection interpolation) then three-dimensional tracers, in that block order.
// groups: counts[g], xyOnly[g], interp[g] (0 linear, 1 spline), tolH[g] (x, y
// blocks), tolV[g] (z block); x, y, z concatenated over groups (z is the fixed
// depth of xy-only particles).  tracers: antialias[i], tolT[i].
int wvref_system_create(const std::uint64_t* sizes, const double* values, const std::uint8_t* flags, int schedule,
                        int nGroups, const int* counts, const int* xyOnly, const int* interp, const double* tolH,
                        const double* tolV, const double* x, const double* y, const double* z, int nTracers,
                        const int* antialias, const double* tolT, void** out) {
    *out = nullptr;
    auto h = std::make_unique<RefSystem>();
    const auto c = makeConfiguration(sizes, values, flags);
    WVTransformConstantStratificationDescriptor transform;
    auto status = WVTransformConstantStratificationDescriptor::create(c, transform);
    if (!status) return static_cast<int>(status.code);
    h->M = transform.spectralShape().elementCount();
    WVPortableObserverRecord record;
    const std::vector<std::size_t> shape{c.Nj, transform.Nkl()};
    for (const char* name : {"Ap", "Am", "A0"})
        record.stateBlocks.push_back({name, WVStateScalarType::complex64, shape, WVToleranceKind::coefficientEnergyScaled,
                                      1e-6, WVStateOwnership::integratorOwned, WVRestartRequirement::requiredDynamicState});
    auto addReal = [&](const std::string& name, std::vector<std::size_t> dims, double tol) {
        record.stateBlocks.push_back({name, WVStateScalarType::real64, std::move(dims), WVToleranceKind::uniformAbsolute,
                                      tol, WVStateOwnership::integratorOwned, WVRestartRequirement::requiredDynamicState});
    };
    WVObserverRecord coefficients;
    coefficients.identifier = "coefficients";
    coefficients.name = "Wave-vortex coefficients";
    coefficients.typeIdentifier = "WVCoefficients";
    coefficients.stateBlockIdentifiers = {"Ap", "Am", "A0"};
    record.observers.push_back(coefficients);
    std::size_t off = 0;
    for (int g = 0; g < nGroups; ++g) {
        const std::string id = "particles" + std::to_string(g);
        const std::size_t n = static_cast<std::size_t>(counts[g]);
        addReal(id + "-x", {n}, tolH[g]);
        addReal(id + "-y", {n}, tolH[g]);
        if (!xyOnly[g]) addReal(id + "-z", {n}, tolV[g]);
        WVObserverRecord o;
        o.identifier = id;
        o.name = id;
        o.typeIdentifier = "WVLagrangianParticles";
        o.stateBlockIdentifiers = {id + "-x", id + "-y"};
        if (!xyOnly[g]) o.stateBlockIdentifiers.push_back(id + "-z");
        o.x.assign(x + off, x + off + n);
        o.y.assign(y + off, y + off + n);
        o.z.assign(z + off, z + off + n);
        o.isXYOnly = xyOnly[g] != 0;
        o.advectionInterpolation = interp[g] ? WVPositionInterpolation::spline : WVPositionInterpolation::linear;
        o.trackedFieldInterpolation = WVPositionInterpolation::linear;
        o.fieldNames = {"u"};
        o.horizontalAbsoluteTolerance = tolH[g];
        o.verticalAbsoluteTolerance = tolV[g];
        record.observers.push_back(o);
        off += n;
    }
    for (int i = 0; i < nTracers; ++i) {
        const std::string id = "tracer" + std::to_string(i);
        addReal(id, {c.Nx, c.Ny, c.Nz}, tolT[i]);
        WVObserverRecord o;
        o.identifier = id;
        o.name = id;
        o.typeIdentifier = "WVTracer";
        o.stateBlockIdentifiers = {id};
        o.shouldAntialias = antialias[i] != 0;
        record.observers.push_back(o);
    }
    std::shared_ptr<const WVExtensionCatalog> catalog;
    status = makeBuiltInExtensionCatalog(catalog);
    if (!status) return static_cast<int>(status.code);
    WVPortableObserverDescriptor descriptor;
    status = WVPortableObserverDescriptor::create(record, catalog, descriptor);
    if (!status) { h->message = status.message; *out = h.release(); return static_cast<int>(status.code); }
    WVFrozenForcingSchedule frozen;
    frozen.entries.push_back(forcingEntry("WVNonlinearAdvection", "nonlinear", WVForcingStage::spatial, 127));
    if (schedule == 1) frozen.entries.push_back(forcingEntry("WVAdaptiveDamping", "adaptive", WVForcingStage::spectral, 100));
    status = WVConstantStratificationIntegrationSystem::create(c, frozen, descriptor, catalog,
                                                               std::make_unique<WVReferenceFFTEngine>(), h->system);
    if (!status) { h->message = status.message; *out = h.release(); return static_cast<int>(status.code); }
    *out = h.release();
    return 0;
}

void wvref_system_destroy(void* s) { delete static_cast<RefSystem*>(s); }
const char* wvref_system_message(void* s) { return s ? static_cast<RefSystem*>(s)->message.c_str() : ""; }

// Number of doubles in the packed additional state.
std::uint64_t wvref_system_extra(void* s) {
    std::uint64_t n = 0;
    for (const auto& b : static_cast<RefSystem*>(s)->system->stateLayout().additionalBlocks()) n += b.elementCount;
    return n;
}

// evaluateRightHandSide on (Ap, Am, A0, extra) -> (Fp, Fm, F0, extraRhs).
int wvref_system_rhs(void* sp, double t, double t0, double* Ap, double* Am, double* A0, double* extra, double* Fp,
                     double* Fm, double* F0, double* extraRhs) {
    auto* h = static_cast<RefSystem*>(sp);
    const auto shape = h->system->stateLayout().coefficientShape();
    auto inViews = blockViews(*h->system, extra);
    auto outViews = blockViews(*h->system, extraRhs);
    WVMutableIntegrationState state{{t, t0, {mview(Ap, shape), mview(Am, shape), mview(A0, shape)}}, inViews.data(),
                                    inViews.size()};
    std::vector<WVAdditionalStateBlockConstView> cviews;
    const auto view = integrationConstView(state, cviews);
    WVIntegrationFlux flux{{mview(Fp, shape), mview(Fm, shape), mview(F0, shape)}, outViews.data(), outViews.size()};
    const auto status = h->system->evaluateRightHandSide(view, flux);
    return status ? 0 : sys_fail(h, status);
}

// WVFixedStepRK4 over the system: steps of dt, state in place, *t advanced.
int wvref_system_rk4(void* sp, double* Ap, double* Am, double* A0, double* extra, double* t, double t0, double dt,
                     int steps) {
    auto* h = static_cast<RefSystem*>(sp);
    const auto shape = h->system->stateLayout().coefficientShape();
    auto views = blockViews(*h->system, extra);
    WVMutableIntegrationState state{{*t, t0, {mview(Ap, shape), mview(Am, shape), mview(A0, shape)}}, views.data(),
                                    views.size()};
    WVFixedStepRK4 rk4(*h->system);
    auto status = rk4.prepareStateAfterRestart(state);
    for (int i = 0; i < steps && status; ++i) status = rk4.step(state, dt);
    if (!status) return sys_fail(h, status);
    *t = state.waveVortex.t;
    return 0;
}

// WVAdaptiveRK23 over the system (options as wvref_rk23_advance; counts =
// {accepted, rejected, rhs evaluations, fsal reuses}).
int wvref_system_rk23(void* sp, const double* opts, double* Ap, double* Am, double* A0, double* extra, double* t,
                      double t0, double finalTime, double initialStep, unsigned long long* counts, double* nextStep,
                      double* steps, int cap) {
    auto* h = static_cast<RefSystem*>(sp);
    const auto shape = h->system->stateLayout().coefficientShape();
    auto views = blockViews(*h->system, extra);
    WVMutableIntegrationState state{{*t, t0, {mview(Ap, shape), mview(Am, shape), mview(A0, shape)}}, views.data(),
                                    views.size()};
    WVAdaptiveRK23Options o;
    o.relativeTolerance = opts[0];
    o.absoluteToleranceScale = opts[1];
    o.safetyFactor = opts[2];
    o.rejectionFloorFactor = opts[3];
    o.maximumStepFactor = opts[4];
    o.maximumStepSize = opts[5];
    WVAdaptiveRK23 rk(*h->system, o);
    auto status = rk.prepareStateAfterRestart(state);
    if (status) status = rk.advanceToTime(state, finalTime, initialStep);
    if (!status) return sys_fail(h, status);
    *t = state.waveVortex.t;
    counts[0] = rk.metrics().acceptedStepCount;
    counts[1] = rk.metrics().rejectedStepCount;
    counts[2] = rk.metrics().rightHandSideEvaluationCount;
    counts[3] = rk.metrics().fsalReuseCount;
    *nextStep = rk.nextStepSize();
    const auto& d = rk.stepDiagnostics();
    for (int i = 0; i < cap && i < static_cast<int>(d.size()); ++i) steps[i] = d[i].acceptedStepSize;
    return 0;
}

// WVFixedStepRK4 with retained dense output: advanceToTime(finalTime, dt) from
// *t, then the interpolant of the last step at denseTime into dense ([3][M]).
int wvref_rk4_dense(void* handle, double* Ap, double* Am, double* A0, double* t, double t0, double finalTime, double dt,
                    double denseTime, double* dense, double* lastInterval) {
    auto* h = static_cast<RefHandle*>(handle);
    const auto s = h->kernel->descriptor().spectralShape();
    WVFixedStepRK4Options o;
    o.retainDenseOutput = true;
    WVFixedStepRK4 rk(*h->system, o);
    WVMutableIntegrationState state{{*t, t0, {mview(Ap, s), mview(Am, s), mview(A0, s)}}, nullptr, 0};
    auto status = rk.prepareStateAfterRestart(state);
    if (status) status = rk.advanceToTime(state, finalTime, dt);
    if (!status) return fail(h, status);
    *t = state.waveVortex.t;
    lastInterval[0] = rk.initialTime();
    lastInterval[1] = rk.finalTime();
    const std::size_t M = s.elementCount();
    WVMutableIntegrationState out{{0.0, t0, {mview(dense, s), mview(dense + 2 * M, s), mview(dense + 4 * M, s)}}, nullptr, 0};
    status = rk.evaluateDenseOutput(denseTime, out);
    return status ? 0 : fail(h, status);
}

} // extern "C"

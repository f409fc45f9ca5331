/*
 * wvgpu.h — C ABI of the GB300 (sm_103a) constant-stratification spectral
 * time step of WaveVortexModel: wave-vortex transforms, the nonlinear flux
 * with 2/3 antialiasing, adaptive damping, fixed-step RK4 (with advanceToTime
 * and dense output) and adaptive RK23; the advection-field flux entries, field
 * and field-family derivatives and F-grid scalar advection; integration
 * systems with Lagrangian particles and tracers; vector-Jacobian products of
 * the flux, the inverse transform and RK4; ensembles of uneven grids in one
 * CUDA graph; FP64, mixed (FP32 + split-BF16 tensor cores) and paired-FP32
 * (FP32X2) arithmetic.
 *
 * Plain pointers and sizes only.  Coefficient arrays are column-major
 * [Nj, Nkl] complex doubles stored as interleaved (re, im) pairs (the
 * reference's WVComplex64 layout, CompiledKernel/include/WaveVortexKernel/
 * WVKernelTypes.hpp:13-20); spatial field bundles are column-major
 * [Nx, Ny, Nz, Nfield] doubles (x fastest).
 *
 * Each entry point names the reference interface it replaces.  Host-pointer
 * entries copy through the handle's device buffers (the drop-in path for the
 * MATLAB gateway and PortableRuntime); *_device entries take device pointers
 * and a cudaStream_t passed as void* (the path for torch / CUDA callers).
 */
#ifndef WVGPU_H
#define WVGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WV_CONTRACT_VERSION 4u /* WVKernelContractVersion, WVKernelTypes.hpp:11 */

/* Numerically identical to wavevortex::WVKernelStatusCode (WVKernelTypes.hpp:22-35). */
enum {
    WV_SUCCESS = 0,
    WV_INVALID_CONFIGURATION = 1,
    WV_INVALID_SHAPE = 2,
    WV_INVALID_POINTER = 3,
    WV_OVERLAPPING_ARRAYS = 4,
    WV_SIZE_OVERFLOW = 5,
    WV_ALLOCATION_FAILURE = 6,
    WV_FFT_PLAN_FAILURE = 7,
    WV_FFT_EXECUTION_FAILURE = 8,
    WV_NUMERICAL_FAILURE = 9,
    WV_UNSUPPORTED_OPERATION = 10,
    WV_REENTRANT_EXECUTION = 11
};

/* WVTransformConstantStratificationConfiguration (WVKernelTypes.hpp:129-146). */
typedef struct wv_config {
    uint32_t contract_version;
    uint64_t Nx, Ny, Nz, Nj;
    double Lx, Ly, Lz;
    double N0, rho0, g;
    double planetary_radius, rotation_rate, latitude;
    uint8_t is_hydrostatic;
    uint8_t should_antialias;
} wv_config;

/* Arithmetic of a handle.  FP64: the plain drop-in, every stage in double.
 * MIXED: FP32 xy transforms and quadratic products, FP64 phases, projections,
 * flux accumulation and RK4 stage accumulation.
 * FP32X2: the xy transforms, products and vertical contractions in paired FP32
 * ("float-float", about 48 significand bits) on the FP32 pipe, FP64 phases,
 * projections and RK4 -- FP64-class flux accuracy without the FP64 pipe.
 * FP32X2 handles serve every entry point (kernel operations, adjoint, ensembles). */
enum { WV_PRECISION_FP64 = 0, WV_PRECISION_MIXED = 1, WV_PRECISION_FP32X2 = 2 };

/* Forcing schedule of the right-hand side (WVFrozenForcingSchedule entries
 * WVNonlinearAdvection and WVAdaptiveDamping, PortableRuntime/src/WVForcingEngine.cpp). */
#define WV_FORCING_NONLINEAR_ADVECTION 1u
#define WV_FORCING_ADAPTIVE_DAMPING 2u

typedef struct wv_handle wv_handle;

/* Sizes derived from a configuration (no GPU needed). */
typedef struct wv_sizes {
    uint64_t Nx, Ny, Nz, Nj, Nkl, NxHalf;
    uint64_t M;              /* Nj * Nkl coefficients per component */
    uint64_t active_rows;    /* half-spectrum rows holding data (retained + Hermitian completion) */
    uint64_t kx_columns;     /* kx columns 0..kx_columns-1 that hold data */
    uint64_t device_bytes;   /* device memory a handle of this configuration allocates (FP64) */
} wv_sizes;

/* Counters of a handle (subset of WVKernelMetrics, WVTransformConstantStratificationKernel.hpp:12-45). */
typedef struct wv_metrics {
    uint64_t nonlinear_flux_calls;
    uint64_t rhs_evaluations;
    uint64_t forward_calls;
    uint64_t inverse_calls;
    uint64_t rk4_steps;
    uint64_t kernel_launches;
    uint64_t device_bytes;
    double last_max_horizontal_speed;
} wv_metrics;

/* ---- configuration and descriptor (host only, no GPU) ---------------------------- */

/* Validates a configuration and reports its sizes.
 * Replaces WVTransformConstantStratificationDescriptor::create validation
 * (CompiledKernel/src/WVKernelTypes.cpp:119-133,196-201) and the MEX "estimate"
 * command (CompiledKernel/adapters/native-fftw/wv_compiled_backend_mex.cpp:225-245). */
int wv_describe(const wv_config* config, wv_sizes* sizes, char* message, size_t message_capacity);

/* Mode set of the descriptor in canonical WV order (WVKernelTypes.cpp:143-166,286-307):
 * kMode/lMode [Nkl] and omega [Nj,Nkl] (any pointer may be NULL). */
int wv_describe_modes(const wv_config* config, int64_t* kMode, int64_t* lMode, double* omega,
                      uint64_t* storage_rows, uint8_t* conjugated);

/* ---- handle lifetime -------------------------------------------------------------- */

/* Replaces WVTransformConstantStratificationKernel::create
 * (CompiledKernel/include/WaveVortexKernel/WVTransformConstantStratificationKernel.hpp:47)
 * and the MEX "create" command (wv_compiled_backend_mex.cpp:247-260).  Builds the
 * descriptor on the host in FP64, uploads it once, and allocates the device arena
 * on the current CUDA device. */
int wv_create(const wv_config* config, int precision, wv_handle** handle);

/* Replaces the MEX "delete" command (wv_compiled_backend_mex.cpp:276-281). */
void wv_destroy(wv_handle* handle);

/* Message of the last failing call on this handle (WVKernelStatus::message). */
const char* wv_last_message(const wv_handle* handle);

int wv_get_sizes(const wv_handle* handle, wv_sizes* sizes);
int wv_get_metrics(const wv_handle* handle, wv_metrics* metrics);

/* Forcing schedule for wv_evaluate_rhs / wv_rk4_*: a bitwise OR of WV_FORCING_*.
 * Default: WV_FORCING_NONLINEAR_ADVECTION (defaultNonlinearAdvectionSchedule,
 * PortableRuntime/src/WVForcingContracts.cpp:118-132). */
int wv_set_forcing(wv_handle* handle, uint32_t forcing_flags);

/* Per-stage device time of the nonlinear flux, summed over instrumented fluxes
 * (the GPU counterpart of WVKernelMetrics' stage seconds,
 * WVTransformConstantStratificationKernel.hpp:31-44). */
typedef struct wv_stage_times {
    double vertical_inverse_ms;   /* phase, field spectra, vertical inverse contraction */
    double y_inverse_ms;          /* inverse FFTs along y */
    double x_products_ms;         /* c2r along x, quadratic products, r2c along x */
    double y_forward_ms;          /* forward FFTs along y */
    double vertical_forward_ms;   /* vertical forward contraction and projection */
    uint64_t fluxes;
} wv_stage_times;

/* setStageInstrumentation (kernel.cpp:570-581): when enabled, each flux records
 * CUDA events between its five stages on its stream and waits for them, adding
 * the elapsed device time to the handle's stage times (reset on enable). */
int wv_set_stage_instrumentation(wv_handle* handle, int enabled);

/* Kernels of the flux's vertical transforms.  No counterpart in the
 * reference.  WV_VERTICAL_CUDA_CORES: the dense folded contractions on the CUDA
 * cores.  WV_VERTICAL_TENSOR_CORES: the dense contractions on the tensor cores
 * (tcgen05.mma, FP32 accumulators in tensor memory): on mixed-precision handles
 * (Nz <= 255) both vertical transforms as split-BF16 GEMMs (three BF16 pieces
 * per operand, six cross products), the forward one with the flux projection
 * fused into its drain; on FP32X2 handles (Nj <= 96) the vertical inverse as
 * exact GEMMs of six 8-bit digit slices per operand (paired-FP32 accuracy);
 * other handles return WV_UNSUPPORTED_OPERATION. */
#define WV_VERTICAL_CUDA_CORES 0
#define WV_VERTICAL_TENSOR_CORES 1
/* Every precision with 3 <= Nz <= 513: the flux's vertical inverse and forward
 * transforms as complex FFTs of length 2 (Nz - 1) of the even / odd extension
 * over z, one per pair of a cosine-family and a sine-family channel (the
 * reference's own REDFT00 / RODFT00 route), in the handle's arithmetic.
 * wv_set_vertical_kernel sets both directions (the forward transform of a
 * handle without a tensor-core forward kernel keeps the dense contraction). */
#define WV_VERTICAL_FFT 2
int wv_set_vertical_kernel(wv_handle* handle, int kind);
/* The kernel of the flux's vertical inverse transform (WV_VERTICAL_*). */
int wv_get_vertical_kernel(const wv_handle* handle, int* kind);
/* Both directions on their own: the inverse (field spectra -> z grid) and the
 * forward (products -> flux coefficients) transform, each any kind the handle
 * has (the tensor-core forward transform: mixed handles with Nz <= 255).  The
 * defaults are the measured fastest: FFTs wherever 3 <= Nz <= 513, except on
 * mixed handles, whose inverse takes the dense contraction below Nz = 97 and
 * forward transform below Nz = 65. */
int wv_set_vertical_kernels(wv_handle* handle, int inverse_kind, int forward_kind);
int wv_get_vertical_kernels(const wv_handle* handle, int* inverse_kind, int* forward_kind);
/* Kernels of the flux's xy FFTs, per axis.  No counterpart in the reference.
 * WV_FFT_REGISTER: register-resident lines of one warp (32 R points, R values
 * per lane, five shuffle butterfly stages; mixed and FP32X2 handles, y lines of
 * 32 R and x rows of 64 R samples for the R each precision has), the default
 * where the length allows; WV_FFT_STOCKHAM: the shared-memory Stockham kernels
 * (every length; the only form of FP64 handles).  The get call reports the
 * kernel that runs. */
#define WV_FFT_REGISTER 0
#define WV_FFT_STOCKHAM 1
int wv_set_fft_variants(wv_handle* handle, int y_variant, int x_variant);
int wv_get_fft_variants(const wv_handle* handle, int* y_variant, int* x_variant);
/* Device status word of the handle (synchronous read): bit 0 is set when a
 * bounded wait inside a kernel ran out (the kernel returned without hanging). */
int wv_get_device_status(wv_handle* handle, unsigned* status);
/* Clears the device status word. */
int wv_reset_device_status(wv_handle* handle);
/* Per-coefficient absolute error tolerances of the adaptive integrator
 * (WVWaveVortexCoefficientErrorPolicy::create, PortableRuntime/src/WVForcingEngine.cpp:79-168):
 * wave[M] for Ap and Am, vortex[M] for A0, [Nj, Nkl] column-major, scaled by
 * absolute_tolerance_scale.  Host memory; no device work. */
int wv_error_tolerances(wv_handle* handle, double absolute_tolerance_scale, double* wave, double* vortex);
int wv_get_stage_times(const wv_handle* handle, wv_stage_times* times);

/* ---- operators (host pointers) ------------------------------------------------------ */

/* WVTransformConstantStratificationKernel::nonlinearFlux (kernel.cpp:1140-1146).
 * Ap, Am, A0 in; Fp, Fm, F0 out; all [Nj, Nkl] complex. */
int wv_nonlinear_flux(wv_handle* handle, double t, double t0,
                      const double* Ap, const double* Am, const double* A0,
                      double* Fp, double* Fm, double* F0);

/* WVIntegrationSystem::evaluateRightHandSide with the handle's forcing schedule
 * (PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:295-330); the
 * MEX "nonlinearFlux" command (wv_compiled_backend_mex.cpp:318-331). */
int wv_evaluate_rhs(wv_handle* handle, double t, double t0,
                    const double* Ap, const double* Am, const double* A0,
                    double* Fp, double* Fm, double* F0);

/* transformUVWEtaToWaveVortex (nonhydrostatic, 4 fields u,v,w,eta) or
 * transformUVEtaToWaveVortex (hydrostatic, 3 fields u,v,eta) (kernel.cpp:583-684);
 * MEX "forward" (wv_compiled_backend_mex.cpp:285-296). */
int wv_forward(wv_handle* handle, const double* fields, double t, double t0,
               double* Ap, double* Am, double* A0);

/* transformWaveVortexToUVWEta (kernel.cpp:686-694,745-776): fields [Nx,Ny,Nz,4];
 * MEX "inverse" (wv_compiled_backend_mex.cpp:297-306). */
int wv_inverse(wv_handle* handle, double t, double t0,
               const double* Ap, const double* Am, const double* A0, double* fields);

/* WVFixedStepRK4::step applied n_steps times (PortableRuntime/src/WVRungeKutta.cpp:335-462)
 * on the handle's forcing schedule.  State updated in place; *t advanced by n_steps*dt. */
int wv_rk4_steps(wv_handle* handle, double* Ap, double* Am, double* A0,
                 double* t, double t0, double dt, int n_steps);

/* ---- operators (device pointers, stream passed as cudaStream_t cast to void*) ------- */

int wv_nonlinear_flux_device(wv_handle* handle, double t, double t0,
                             const double* Ap, const double* Am, const double* A0,
                             double* Fp, double* Fm, double* F0, void* stream);
int wv_evaluate_rhs_device(wv_handle* handle, double t, double t0,
                           const double* Ap, const double* Am, const double* A0,
                           double* Fp, double* Fm, double* F0, void* stream);
int wv_forward_device(wv_handle* handle, const double* fields, double t, double t0,
                      double* Ap, double* Am, double* A0, void* stream);
int wv_inverse_device(wv_handle* handle, double t, double t0,
                      const double* Ap, const double* Am, const double* A0, double* fields, void* stream);
/* ---- adjoint (vector-Jacobian products) --------------------------------------------
 * No counterpart in the reference.  For complex arrays the inner product is
 * <a, b> = Re sum conj(a) b; a cotangent x_bar of an output x is mapped to the
 * cotangent of the inputs such that <x_bar, dx> = <in_bar, d in> for every
 * perturbation.  Device pointers, [Nj, Nkl] complex unless stated.  The first
 * adjoint call on a handle allocates its adjoint workspace.  The nonlinear
 * advection schedule only (adaptive damping's max|u_h| is not differentiable):
 * handles with adaptive damping enabled return WV_UNSUPPORTED_OPERATION. */

/* Flux VJP at state (Ap, Am, A0, t): (Fpb, Fmb, F0b) -> (Apb, Amb, A0b). */
int wv_flux_vjp_device(wv_handle* handle, double t, double t0,
                       const double* Ap, const double* Am, const double* A0,
                       const double* Fpb, const double* Fmb, const double* F0b,
                       double* Apb, double* Amb, double* A0b, void* stream);
/* Inverse-transform VJP: fields_bar [Nx,Ny,Nz,4] -> (Apb, Amb, A0b). */
int wv_inverse_vjp_device(wv_handle* handle, double t, double t0, const double* fields_bar,
                          double* Apb, double* Amb, double* A0b, void* stream);
/* One RK4 step's VJP at state (Ap, Am, A0, t): (Apb, Amb, A0b) hold the cotangent
 * of the state after the step on entry and of the state before it on return.
 * The stage states are recomputed. */
int wv_rk4_step_vjp_device(wv_handle* handle, const double* Ap, const double* Am, const double* A0,
                           double t, double t0, double dt, double* Apb, double* Amb, double* A0b, void* stream);
/* Adjoint of n_steps RK4 steps from state (Ap, Am, A0, t): a forward pass keeps
 * a checkpoint every checkpoint_every steps, each segment is recomputed from its
 * checkpoint and stepped backward.  (Apb, Amb, A0b): cotangent at t + n_steps*dt
 * on entry, at t on return. */
int wv_rk4_adjoint_device(wv_handle* handle, const double* Ap, const double* Am, const double* A0,
                          double t, double t0, double dt, int n_steps, int checkpoint_every,
                          double* Apb, double* Amb, double* A0b, void* stream);

/* Nonlinear flux that allocates no device memory.  No counterpart in the
 * reference: the reference's kernel owns a heap scratch arena.  It exists for
 * callers that cannot call cudaMalloc at the point where they need a flux: a
 * host application whose memory manager owns every device allocation and
 * forbids further driver allocations, or latency-sensitive loops where
 * cudaMalloc's implicit device synchronization is not acceptable.  Inputs and
 * outputs are device pointers supplied by the caller, exactly as for
 * wv_nonlinear_flux_device (no adaptive damping); the handle must already exist
 * (wv_create allocates) and hold a single state, else WV_UNSUPPORTED_OPERATION.
 * The launches and the vertical-kernel choice (wv_set_vertical_kernel) are
 * those of wv_nonlinear_flux_device on the same handle; only the scratch differs.
 * The flux pipeline's scratch lives in one file-scope __device__ array of
 * WV_STATIC_SCRATCH_BYTES, held by every GPU that loads the library until exit.
 * Configurations whose scratch exceeds it are rejected with WV_SIZE_OVERFLOW.
 * The first call on a device looks up the array's device address and keeps it
 * for the process; make that first call before any stream capture.  A device
 * reset (cudaDeviceReset) invalidates the kept address: do not call this entry
 * on a device that was reset after its first call.  All calls share the one
 * array, which keeps the last call's contents, so calls that overlap on the GPU
 * (other streams, other handles) race. */
#define WV_STATIC_SCRATCH_BYTES (32ull << 20)
int wv_nonlinear_flux_device_noalloc(wv_handle* handle, double t, double t0,
                                     const double* Ap, const double* Am, const double* A0,
                                     double* Fp, double* Fm, double* F0, void* stream);

/* nonlinearFluxWithAdvectionFields (kernel.cpp:1148-1158): the flux and the
 * advecting velocity (u, v, w) it used, fields [Nx, Ny, Nz, 3] (x fastest).
 * nonlinearFluxUsingAdvectionFields (kernel.cpp:1160-1171): the flux with the
 * given (u, v, w) as the advecting velocity (the derivatives of the advected
 * fields still come from the state).  transformWaveVortexToUVW (kernel.cpp:696-717):
 * (u, v, w) only.  Host- and device-pointer forms; the fields must not overlap
 * the state or flux arrays (WV_OVERLAPPING_ARRAYS). */
int wv_nonlinear_flux_with_advection_fields(wv_handle* handle, double t, double t0,
                                            const double* Ap, const double* Am, const double* A0,
                                            double* Fp, double* Fm, double* F0, double* fields);
int wv_nonlinear_flux_using_advection_fields(wv_handle* handle, double t, double t0,
                                             const double* Ap, const double* Am, const double* A0,
                                             double* Fp, double* Fm, double* F0, const double* fields);
int wv_inverse_uvw(wv_handle* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
                   double* fields);
int wv_nonlinear_flux_with_advection_fields_device(wv_handle* handle, double t, double t0,
                                                   const double* Ap, const double* Am, const double* A0,
                                                   double* Fp, double* Fm, double* F0, double* fields, void* stream);
int wv_nonlinear_flux_using_advection_fields_device(wv_handle* handle, double t, double t0,
                                                    const double* Ap, const double* Am, const double* A0,
                                                    double* Fp, double* Fm, double* F0, const double* fields, void* stream);
int wv_inverse_uvw_device(wv_handle* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
                          double* fields, void* stream);

/* transformStateFieldDerivatives (kernel.cpp:719-743): (d/dx, d/dy, d/dz) of
 * field 0..3 (u, v, w, eta) at the state, out [Nx, Ny, Nz, 3]. */
int wv_field_derivatives(wv_handle* handle, double t, double t0, const double* Ap, const double* Am, const double* A0,
                         int field, double* out);
int wv_field_derivatives_device(wv_handle* handle, double t, double t0, const double* Ap, const double* Am,
                                const double* A0, int field, double* out, void* stream);

/* transformToSpatialDomainWith{F,G}AllDerivatives (kernel.cpp:819-863): value and
 * (d/dx, d/dy, d/dz) of the F (ffamily = 1) or G (ffamily = 0) field family of
 * (Apm, A0) [Nj, Nkl] complex, fields [Nx, Ny, Nz, 4]. */
int wv_family_derivatives(wv_handle* handle, int ffamily, const double* Apm, const double* A0, double* fields);
int wv_family_derivatives_device(wv_handle* handle, int ffamily, const double* Apm, const double* A0, double* fields,
                                 void* stream);

/* advectFGridScalar (kernel.cpp:1032-1138): rhs = -(u ds/dx + v ds/dy + w ds/dz)
 * of an F-grid scalar s [Nx, Ny, Nz] advected by fields (u, v, w) [Nx, Ny, Nz, 3],
 * spectral derivatives on the full half spectrum; with antialias set, rhs is
 * filtered to the transform's (2/3-disk) rows.  The first call allocates the
 * scalar pipeline's descriptor and scratch. */
int wv_advect_fgrid_scalar(wv_handle* handle, const double* scalar, const double* fields, int antialias, double* rhs);
int wv_advect_fgrid_scalar_device(wv_handle* handle, const double* scalar, const double* fields, int antialias,
                                  double* rhs, void* stream);

/* Runs n_steps RK4 steps on device-resident state; the time is kept on the host
 * (t in/out) exactly as WVFixedStepRK4 advances it (t <- t + dt per step). */
int wv_rk4_steps_device(wv_handle* handle, double* Ap, double* Am, double* A0,
                        double* t, double t0, double dt, int n_steps, void* stream);
/* WVFixedStepRK4Options::retainDenseOutput (PortableRuntime/include/WaveVortexRuntime/
 * WVRungeKutta.hpp:52-54): when enabled, every RK4 entry keeps the last step's end
 * states and first and fourth stage derivatives on the device. */
int wv_rk4_set_dense_output(wv_handle* handle, int enabled);
/* WVFixedStepRK4::advanceToTime (PortableRuntime/src/WVRungeKutta.cpp:464-480): steps of
 * min(dt, final_time - t) until final_time; *t ends at final_time. */
int wv_rk4_advance_to_time_device(wv_handle* handle, double* Ap, double* Am, double* A0, double* t, double t0,
                                  double final_time, double dt, void* stream);
int wv_rk4_advance_to_time(wv_handle* handle, double* Ap, double* Am, double* A0, double* t, double t0,
                           double final_time, double dt);
/* WVFixedStepRK4::evaluateDenseOutput (WVRungeKutta.cpp:482-541): the state at `time`
 * inside the last step (cubic Hermite), written to device arrays. */
int wv_rk4_dense_output_device(wv_handle* handle, double time, double* Ap, double* Am, double* A0, void* stream);

/* ---- ensembles ------------------------------------------------------------------------
 * No counterpart in the reference, which steps one state per kernel object
 * (a caller would hold one WVTransformConstantStratificationKernel per member).
 * An ensemble holds n_groups grids; group g steps members[g] states of
 * group_configs[g] side by side (each stage kernel covers all members of the group in
 * one launch).  wv_ensemble_rk4_device captures the n-step RK4 integration of
 * every group (one stream per group) into one CUDA graph and launches it once;
 * a later call with the same groups and step count updates the graph's
 * parameters instead of capturing anew.  Nonlinear advection schedule.  With
 * autotune set, creation times each group's flux with every FFT variant its grid
 * has (warp-register or shared-memory Stockham, per axis) and keeps the fastest. */
typedef struct wv_ensemble wv_ensemble;
#define WV_ENSEMBLE_MAX_GROUPS 16
#define WV_ENSEMBLE_MAX_CANDIDATES 12
typedef struct wv_ensemble_tuning {
    int warp_y_available, warp_x_available;  /* variants the grid has */
    int tensor_vertical_available;
    int stockham_y, stockham_x;              /* chosen: 1 = Stockham, 0 = warp (where available) */
    int vertical;                            /* chosen kernel of the vertical inverse transform (WV_VERTICAL_*) */
    int vertical_forward;                    /* ... and of the vertical forward transform */
    int candidates;                          /* (y, x) variants timed */
    float candidate_ms[WV_ENSEMBLE_MAX_CANDIDATES]; /* flux time of each (y, x) variant, y outer, ms */
    float vertical_inverse_ms[3];            /* mixed groups: stage time per flux of each vertical kernel
                                                (index WV_VERTICAL_*), -1 where the grid has none */
    float vertical_forward_ms[3];
    float flux_ms;                           /* chosen variant, ms per flux of the whole group */
} wv_ensemble_tuning;
typedef struct wv_ensemble_metrics {
    uint64_t graph_captures, graph_instantiations, graph_updates, graph_launches;
    uint64_t kernel_launches;                /* kernel nodes replayed */
    uint64_t member_steps;
    uint64_t device_bytes;
} wv_ensemble_metrics;
int wv_ensemble_create(const wv_config* group_configs, const int* members, int n_groups, int precision, int autotune,
                       wv_ensemble** ensemble);
void wv_ensemble_destroy(wv_ensemble* ensemble);
const char* wv_ensemble_last_message(const wv_ensemble* ensemble);
int wv_ensemble_get_sizes(const wv_ensemble* ensemble, int group, wv_sizes* sizes);  /* per member */
int wv_ensemble_get_tuning(const wv_ensemble* ensemble, int group, wv_ensemble_tuning* tuning);
int wv_ensemble_get_metrics(const wv_ensemble* ensemble, wv_ensemble_metrics* metrics);
/* Vertical-transform kernel of every group (as wv_set_vertical_kernel); overrides the autotuner. */
int wv_ensemble_set_vertical_kernel(wv_ensemble* ensemble, int kind);
/* states[g]: device array [members[g]][3][Nkl][Nj] complex (each member's Ap, Am,
 * A0 back to back), advanced in place.  t[g] (in/out) is group g's time and
 * dt[g] its step; on return t[g] has advanced by n_steps steps of dt[g]. */
int wv_ensemble_rk4_device(wv_ensemble* ensemble, double* const* states, double* t, double t0, const double* dt,
                           int n_steps, void* stream);

/* ---- adaptive RK23 ---------------------------------------------------------------------
 * WVAdaptiveRK23 (PortableRuntime/include/WaveVortexRuntime/WVRungeKutta.hpp:112-196,
 * PortableRuntime/src/WVRungeKutta.cpp:554-983): Bogacki-Shampine 3(2) pair with
 * first-same-as-last reuse and the "matlab-ode23-v1" step-size controller, over the
 * handle's scheduled right-hand side (wv_evaluate_rhs).  Stage states, derivatives and
 * the error norm stay on the device; the controller reads one double per attempt. */
typedef struct wv_rk23 wv_rk23;
/* WVAdaptiveRK23Options (WVRungeKutta.hpp:112-120). */
typedef struct wv_rk23_options {
    double relative_tolerance;                  /* 1e-3 */
    double absolute_tolerance_scale;            /* 1e-6: scales the per-coefficient energy tolerances */
    double safety_factor;                       /* 0.8 */
    double rejection_floor_factor;              /* 0.5 */
    double maximum_step_factor;                 /* 5 */
    double maximum_step_size;                   /* +inf */
    uint64_t maximum_recorded_step_diagnostics; /* 512 */
} wv_rk23_options;
/* WVAdaptiveRK23StepDiagnostic (WVRungeKutta.hpp:122-130). */
typedef struct wv_rk23_step_diagnostic {
    double initial_time;
    double accepted_step_size;
    double normalized_error;
    double next_step_size;
    uint64_t rejected_attempt_count;
    uint64_t rhs_evaluation_count;
    uint8_t reused_fsal_derivative;
} wv_rk23_step_diagnostic;
/* The RK23 fields of WVIntegratorMetrics (WVRungeKutta.hpp:14-50). */
typedef struct wv_rk23_metrics {
    uint64_t rhs_evaluations;
    uint64_t accepted_steps;
    uint64_t rejected_steps;
    uint64_t fsal_reuses;
    uint64_t fsal_invalidations;
    uint64_t rejected_initial_derivative_reuses;
    uint64_t dense_output_evaluations;
    double last_proposed_step_size;
    double last_accepted_step_size;
    double normalized_error;
    double next_step_size;
    uint64_t workspace_bytes;
} wv_rk23_metrics;
void wv_rk23_default_options(wv_rk23_options* options);
/* Binds an integrator to a handle (the handle must outlive it).  Builds the absolute
 * tolerances (WVWaveVortexCoefficientErrorPolicy, PortableRuntime/src/WVForcingEngine.cpp:79-168)
 * and allocates five state-sized device buffers. */
int wv_rk23_create(wv_handle* handle, const wv_rk23_options* options, wv_rk23** integrator);
void wv_rk23_destroy(wv_rk23* integrator);
const char* wv_rk23_last_message(const wv_rk23* integrator);
/* prepareStateAfterRestart (WVRungeKutta.cpp:645-657): forgets the stored derivative,
 * the accepted step and the diagnostics. */
int wv_rk23_prepare_after_restart(wv_rk23* integrator);
/* WVAdaptiveRK23::step on device-resident state (each [Nj, Nkl] complex), updated in
 * place; *t advances by the accepted step.  Synchronizes the stream once per attempt. */
int wv_rk23_step_device(wv_rk23* integrator, double* Ap, double* Am, double* A0, double* t, double t0,
                        double proposed_step, void* stream);
/* WVAdaptiveRK23::advanceToTime (WVRungeKutta.cpp:892-912); *t ends at final_time. */
int wv_rk23_advance_to_time_device(wv_rk23* integrator, double* Ap, double* Am, double* A0, double* t, double t0,
                                   double final_time, double initial_step, void* stream);
/* Host-pointer form of wv_rk23_advance_to_time_device. */
int wv_rk23_advance_to_time(wv_rk23* integrator, double* Ap, double* Am, double* A0, double* t, double t0,
                            double final_time, double initial_step);
/* WVAdaptiveRK23::evaluateDenseOutput (WVRungeKutta.cpp:914-981) into device arrays. */
int wv_rk23_dense_output_device(wv_rk23* integrator, double time, double* Ap, double* Am, double* A0, void* stream);
int wv_rk23_next_step_size(const wv_rk23* integrator, double* next_step_size);
/* Interval of the last accepted step; WV_UNSUPPORTED_OPERATION when there is none. */
int wv_rk23_last_accepted_step(const wv_rk23* integrator, double* initial_time, double* final_time);
int wv_rk23_get_metrics(const wv_rk23* integrator, wv_rk23_metrics* metrics);
/* Copies up to capacity recorded diagnostics; *count receives the number recorded. */
int wv_rk23_get_diagnostics(const wv_rk23* integrator, wv_rk23_step_diagnostic* diagnostics, uint64_t capacity,
                            uint64_t* count);
/* Audit hash of the absolute tolerances (WVAdaptiveRK23::toleranceHash, WVRungeKutta.cpp:26-37,
 * 602-613): FNV-1a over the doubles rounded to 32 significand bits; component_hashes
 * receives the three per-component hashes (A+, A-, A0) when not NULL. */
int wv_rk23_tolerance_hash(const wv_rk23* integrator, uint64_t* hash, uint64_t* component_hashes);

/* ---- integration system with integrated observers ---------------------------------------
 * WVConstantStratificationIntegrationSystem with Lagrangian particles and three-dimensional
 * tracers (PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:112-400): one
 * scheduled flux per right-hand side also yields the advection fields (u, v, w), which every
 * tracer (advectFGridScalar) and every particle group (velocity at the particle positions)
 * shares.  The packed state is Ap, Am, A0 ([Nj, Nkl] complex each) followed by the additional
 * blocks in order: for each particle group x, y[, z] (count doubles each; x and y unwrapped,
 * periodicity applied only when sampling), then for each tracer a [Nx, Ny, Nz] field. */
typedef struct wv_system wv_system;
/* WVPositionInterpolation (PortableRuntime/include/WaveVortexRuntime/WVObserverContracts.hpp:32). */
#define WV_INTERPOLATION_LINEAR 0
#define WV_INTERPOLATION_SPLINE 1
/* WVLagrangianParticles (WVLagrangianParticles.hpp): one particle group. */
typedef struct wv_particle_group {
    uint64_t count;
    int xy_only;                 /* x, y blocks only; depth fixed per particle */
    int interpolation;           /* WV_INTERPOLATION_* for the advecting velocity */
    const double* z_fixed;       /* host [count]: depths of xy-only particles (NULL otherwise) */
    double horizontal_tolerance; /* absolute tolerance of the x and y blocks (adaptive RK23) */
    double vertical_tolerance;   /* absolute tolerance of the z block */
} wv_particle_group;
/* WVTracer (WVTracer.hpp): one three-dimensional tracer. */
typedef struct wv_tracer {
    int antialias;               /* shouldAntialias of the tracer's scalar advection */
    double absolute_tolerance;
} wv_tracer;
/* Binds a system to a handle (which must outlive it); the handle's forcing schedule applies. */
int wv_system_create(wv_handle* handle, const wv_particle_group* groups, int n_groups, const wv_tracer* tracers,
                     int n_tracers, wv_system** system);
void wv_system_destroy(wv_system* system);
const char* wv_system_last_message(const wv_system* system);
/* Doubles of the packed state, and offset / length (in doubles) of each additional block. */
int wv_system_get_layout(const wv_system* system, uint64_t* state_doubles, uint64_t* n_blocks, uint64_t* offsets,
                         uint64_t* lengths, uint64_t capacity);
/* evaluateRightHandSide (WVConstantStratificationIntegrationSystem.cpp:295-400) on packed
 * device arrays. */
int wv_system_rhs_device(wv_system* system, double t, double t0, const double* state, double* rhs, void* stream);
/* WVFixedStepRK4::step over the packed state, n_steps times (device and host forms). */
int wv_system_rk4_device(wv_system* system, double* state, double* t, double t0, double dt, int n_steps, void* stream);
int wv_system_rk4(wv_system* system, double* state, double* t, double t0, double dt, int n_steps);
/* Adaptive RK23 over a system's packed state: the additional blocks enter the error norm with
 * their absolute tolerances (UnifiedErrorPolicy, WVConstantStratificationIntegrationSystem.cpp:47-86). */
int wv_rk23_create_for_system(wv_system* system, const wv_rk23_options* options, wv_rk23** integrator);
int wv_rk23_system_step_device(wv_rk23* integrator, double* state, double* t, double t0, double proposed_step,
                               void* stream);
int wv_rk23_system_advance_to_time_device(wv_rk23* integrator, double* state, double* t, double t0, double final_time,
                                          double initial_step, void* stream);
int wv_rk23_system_dense_output_device(wv_rk23* integrator, double time, double* state, void* stream);

/* ---- test hooks ----------------------------------------------------------------------
 * No counterpart in the reference's C ABI.  The reference's contract tests
 * inject plan, allocation and execution failures through a failing FFT engine
 * (tools/compiled-kernel/tests/TestWVKernelContract.cpp:153-175,331-355); these
 * hooks give the GPU library's tests the same reach, on the host, without a
 * GPU fault.  Not for production use. */
/* The library's next n device allocations for handles succeed and the one after
 * fails as cudaErrorMemoryAllocation would (n < 0: off; one-shot). */
int wv_test_fail_allocation_after(long long n);
/* Device bytes held by all live handles of this process. */
long long wv_test_live_device_bytes(void);
/* The handle's next n flux launch sequences run and the one after fails before
 * launching anything, reported as WV_FFT_EXECUTION_FAILURE with the message
 * "...: injected execution failure" (n < 0: off; one-shot). */
int wv_test_fail_launch_after(wv_handle* handle, long long n);
/* hold != 0 marks the handle as inside an operation, so every entry returns
 * WV_REENTRANT_EXECUTION until it is released with hold = 0. */
int wv_test_hold_busy(wv_handle* handle, int hold);
/* polls != 0: the tensor-core vertical inverse (k_vinv_tc) waits for its first
 * matrix operand without the copy being issued, at most `polls` times; the wait
 * runs out before any MMA, the kernel sets bit 0 of the device status word,
 * frees its tensor memory and returns (the flux's output is then undefined).
 * polls = 0 restores normal operation. */
int wv_test_inject_wait_timeout(wv_handle* handle, unsigned polls);

#ifdef __cplusplus
}
#endif

#endif /* WVGPU_H */

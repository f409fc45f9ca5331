// Adaptive RK23 on the device (include/wvgpu.h, wv_rk23_*): WVAdaptiveRK23
// (PortableRuntime/src/WVRungeKutta.cpp:554-983) with the stage states, the
// four stage derivatives and the embedded error norm resident in HBM.  The
// step-size controller (wv_rk23_controller.hpp) runs on the host and reads one
// double per attempt: the max-reduced normalized error.
//
// Stage arithmetic follows IntegrationBuffer::setAffine / addScaled /
// setWeightedCandidate (WVRungeKutta.cpp:140-184) operation for operation,
// without contraction.  The right-hand side is the handle's scheduled flux
// (wv_evaluate_rhs_device) on the stage buffer, or the right-hand side of an
// integration system (wv_system_*) whose packed state adds real blocks
// (particles, tracers) with uniform absolute tolerances.
#include "wvgpu.h"
#include "wv_descriptor.hpp"
#include "wv_internal.hpp"
#include "wv_rk23_controller.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

namespace wvgpu {
namespace dev {

// A state: the three coefficient arrays (A+, A-, A0), each 2 M doubles, and
// optionally the additional real blocks of an integration system (n[3]
// doubles).  Derivative and stage buffers are packed in that order.
struct State4 {
    const double* p[4];
    size_t n[4];
};
struct MutState4 {
    double* p[4];
};

// Offset of component c in a packed buffer.
__device__ __forceinline__ size_t packed_offset(const State4& s, int c) {
    size_t o = 0;
    for (int i = 0; i < c; ++i) o += s.n[i];
    return o;
}

// stage = base + scale * k ; grid.y = component
__global__ void k_rk23_affine(State4 base, const double* __restrict__ k, double scale, double* __restrict__ stage) {
    const int c = blockIdx.y;
    const double* b = base.p[c];
    const size_t o = packed_offset(base, c), n = base.n[c];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        stage[o + i] = __dadd_rn(b[i], __dmul_rn(scale, k[o + i]));
}

// stage = ((base + s1 k1) + s2 k2) + s3 k3
__global__ void k_rk23_candidate(State4 base, const double* __restrict__ k1, const double* __restrict__ k2,
                                 const double* __restrict__ k3, double s1, double s2, double s3, double* __restrict__ stage) {
    const int c = blockIdx.y;
    const double* b = base.p[c];
    const size_t o = packed_offset(base, c), n = base.n[c];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v = __dadd_rn(b[i], __dmul_rn(s1, k1[o + i]));
        v = __dadd_rn(v, __dmul_rn(s2, k2[o + i]));
        stage[o + i] = __dadd_rn(v, __dmul_rn(s3, k3[o + i]));
    }
}

__device__ __forceinline__ double rk23_error_component(double h, double a1, double a2, double a3, double a4) {
    constexpr double b1 = 2.0 / 9.0 - 7.0 / 24.0, b2 = 1.0 / 3.0 - 0.25, b3 = 4.0 / 9.0 - 1.0 / 3.0;
    return __dmul_rn(h, __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(b1, a1), __dmul_rn(b2, a2)), __dmul_rn(b3, a3)), __dmul_rn(0.125, a4)));
}

// Embedded error of the Bogacki-Shampine pair, normalized per coefficient
// (WVRungeKutta.cpp:760-840) and max-reduced into *errBits (the bit pattern of
// a nonnegative double orders like the double).  grid.y = component: 0-2 the
// complex coefficients with tolerances tolWave (A+, A-) / tolVortex (A0), one
// complex value per iteration; 3 the real blocks with per-element tolerances.
__global__ void __launch_bounds__(256) k_rk23_error(State4 base, const double* __restrict__ stage, const double* __restrict__ k1,
                                                   const double* __restrict__ k2, const double* __restrict__ k3,
                                                   const double* __restrict__ k4, double h, double relTol,
                                                   const double* __restrict__ tolWave, const double* __restrict__ tolVortex,
                                                   const double* __restrict__ tolExtra, unsigned long long* __restrict__ errBits) {
    const int c = blockIdx.y;
    const double* y0 = base.p[c];
    const size_t o = packed_offset(base, c);
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    double worst = 0.0;
    if (c < 3) {
        const double* tol = c < 2 ? tolWave : tolVortex;
        const size_t M = base.n[c] / 2;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < M; i += (size_t)gridDim.x * blockDim.x) {
            const size_t r = o + 2 * i, im = r + 1;
            const double er = rk23_error_component(h, k1[r], k2[r], k3[r], k4[r]);
            const double ei = rk23_error_component(h, k1[im], k2[im], k3[im], k4[im]);
            const double a0 = hypot(y0[2 * i], y0[2 * i + 1]);
            const double a1 = hypot(stage[r], stage[im]);
            const double scale = fmax(tol[i], __dmul_rn(relTol, fmax(a0, a1)));
            double ratio = hypot(er, ei) / scale;
            if (!isfinite(ratio)) ratio = inf;
            worst = fmax(worst, ratio);
        }
    } else {
        const size_t n = base.n[3];
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
            const double e = rk23_error_component(h, k1[o + i], k2[o + i], k3[o + i], k4[o + i]);
            const double scale = fmax(tolExtra[i], __dmul_rn(relTol, fmax(fabs(y0[i]), fabs(stage[o + i]))));
            double ratio = fabs(e) / scale;
            if (!isfinite(ratio)) ratio = inf;
            worst = fmax(worst, ratio);
        }
    }
    for (int off = 16; off > 0; off >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, off));
    __shared__ double part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = worst;
    __syncthreads();
    if (threadIdx.x == 0) {
        double w = part[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) w = fmax(w, part[i]);
        atomicMax(errBits, static_cast<unsigned long long>(__double_as_longlong(w)));
    }
}

// out = ((((endpoint + (h w0) k1) + (h w1) k2) + (h w2) k3) + (h w3) k4)
__global__ void k_rk23_dense(State4 layout, const double* __restrict__ endpoint, const double* __restrict__ k1,
                             const double* __restrict__ k2, const double* __restrict__ k3, const double* __restrict__ k4,
                             double s0, double s1, double s2, double s3, MutState4 out) {
    const int c = blockIdx.y;
    const size_t o = packed_offset(layout, c), n = layout.n[c];
    double* dst = out.p[c];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double v = __dadd_rn(endpoint[o + i], __dmul_rn(s0, k1[o + i]));
        v = __dadd_rn(v, __dmul_rn(s1, k2[o + i]));
        v = __dadd_rn(v, __dmul_rn(s2, k3[o + i]));
        dst[i] = __dadd_rn(v, __dmul_rn(s3, k4[o + i]));
    }
}

}  // namespace dev

namespace {

// Device side of the controller: buffers, the bound handle (or integration
// system) and the caller's state.
struct DeviceRk23Backend {
    wv_handle* handle = nullptr;
    wv_system* system = nullptr;  // integration system with additional blocks, or null
    size_t M = 0;                 // complex coefficients per component
    size_t nExtra = 0;            // doubles of the system's additional blocks
    double* k[4] = {};            // stage derivatives, packed state each
    double* stage = nullptr;      // stage / candidate / accepted state, packed
    double* tolWave = nullptr;    // [M]
    double* tolVortex = nullptr;  // [M]
    const double* tolExtra = nullptr;  // [nExtra] (the system's)
    unsigned long long* errBits = nullptr;
    double* errHost = nullptr;    // pinned
    double* hostState = nullptr;  // device mirror for the host-pointer entry (allocated on first use)
    // per call
    dev::MutState4 base{};
    double t0 = 0.0;
    cudaStream_t stream = nullptr;
    dev::MutState4 denseOut{};
    std::string msg;

    size_t packed() const { return 6 * M + nExtra; }
    unsigned components() const { return nExtra ? 4u : 3u; }
    unsigned grid_for(size_t n) const { return static_cast<unsigned>(std::min<size_t>((n + 255) / 256, wvgpu::grid_cap(8))); }
    int cuda(cudaError_t e, const char* where) {
        if (e == cudaSuccess) return WV_SUCCESS;
        msg = std::string(where) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_EXECUTION_FAILURE;
    }
    dev::State4 layout_of(const dev::MutState4& s) const {
        return {{s.p[0], s.p[1], s.p[2], s.p[3]}, {2 * M, 2 * M, 2 * M, nExtra}};
    }
    dev::State4 cbase() const { return layout_of(base); }
    // Binds a packed system state (coefficients then additional blocks).
    void bind_packed(dev::MutState4& s, double* packed) const {
        s = {{packed, packed + 2 * M, packed + 4 * M, packed + 6 * M}};
    }

    int rhs(int slot, bool fromStage, double t) {
        const size_t M2 = 2 * M;
        double* out = k[slot];
        if (system) {
            const double* x = fromStage ? stage : base.p[0];  // packed
            const int rc = wvgpu::system_rhs(system, t, t0, x, out, stream);
            if (rc) msg = wv_system_last_message(system);
            return rc;
        }
        const double* x0 = fromStage ? stage : base.p[0];
        const double* x1 = fromStage ? stage + M2 : base.p[1];
        const double* x2 = fromStage ? stage + 2 * M2 : base.p[2];
        const int rc = wv_evaluate_rhs_device(handle, t, t0, x0, x1, x2, out, out + M2, out + 2 * M2, stream);
        if (rc) msg = wv_last_message(handle);
        return rc;
    }
    int affine(int slot, double scale) {
        dev::k_rk23_affine<<<dim3(grid_for(2 * M), components()), 256, 0, stream>>>(cbase(), k[slot], scale, stage);
        return cuda(cudaGetLastError(), "RK23 stage state");
    }
    int candidate(double s1, double s2, double s3) {
        dev::k_rk23_candidate<<<dim3(grid_for(2 * M), components()), 256, 0, stream>>>(cbase(), k[0], k[1], k[2], s1, s2, s3, stage);
        return cuda(cudaGetLastError(), "RK23 candidate");
    }
    int error(double h, double relTol, double* e) {
        int rc = cuda(cudaMemsetAsync(errBits, 0, sizeof(unsigned long long), stream), "RK23 error norm");
        if (rc) return rc;
        dev::k_rk23_error<<<dim3(grid_for(M), components()), 256, 0, stream>>>(cbase(), stage, k[0], k[1], k[2], k[3], h, relTol,
                                                                               tolWave, tolVortex, tolExtra, errBits);
        rc = cuda(cudaGetLastError(), "RK23 error norm");
        if (rc) return rc;
        rc = cuda(cudaMemcpyAsync(errHost, errBits, sizeof(double), cudaMemcpyDeviceToHost, stream), "RK23 error norm");
        if (rc) return rc;
        rc = cuda(cudaStreamSynchronize(stream), "RK23 error norm");
        if (rc) return rc;
        *e = *errHost;
        return WV_SUCCESS;
    }
    int accept() {
        const auto l = cbase();
        size_t o = 0;
        for (unsigned c = 0; c < components(); ++c) {
            const int rc = cuda(cudaMemcpyAsync(base.p[c], stage + o, l.n[c] * sizeof(double), cudaMemcpyDeviceToDevice, stream),
                                "RK23 accept");
            if (rc) return rc;
            o += l.n[c];
        }
        return WV_SUCCESS;
    }
    void swap_first_last() { std::swap(k[0], k[3]); }
    int dense(double h, const double w[4]) {
        dev::k_rk23_dense<<<dim3(grid_for(2 * M), components()), 256, 0, stream>>>(
            layout_of(denseOut), stage, k[0], k[1], k[2], k[3], h * w[0], h * w[1], h * w[2], h * w[3], denseOut);
        return cuda(cudaGetLastError(), "RK23 dense output");
    }
    std::string message() const { return msg; }
};

uint64_t hash_tolerance(uint64_t hash, double value) {
    uint64_t bits = 0;
    std::memcpy(&bits, &value, sizeof(bits));
    bits = (bits + UINT64_C(0x80000)) & ~UINT64_C(0xfffff);  // keep about 32 significand bits
    hash ^= bits;
    return hash * UINT64_C(1099511628211);
}

}  // namespace
}  // namespace wvgpu

struct wv_rk23 {
    wvgpu::DeviceRk23Backend backend;
    wvgpu::Rk23Controller<wvgpu::DeviceRk23Backend> controller;
    wv_rk23_options options;
    std::string message;
    uint64_t hash = 0, componentHash[3] = {};
    size_t workspaceBytes = 0;
    std::atomic<bool> busy{false};
    explicit wv_rk23(const wv_rk23_options& o) : controller(backend, o), options(o) {}
};

namespace {

int rk_fail(wv_rk23* r, int code, const std::string& m) {
    if (r) r->message = m;
    return code;
}

struct BusyGuard {
    std::atomic<bool>& flag;
    bool entered;
    explicit BusyGuard(std::atomic<bool>& f) : flag(f), entered(!f.exchange(true)) {}
    ~BusyGuard() { if (entered) flag.store(false); }
};

void release(wv_rk23* r) {
    auto& b = r->backend;
    for (double*& p : b.k) { if (p) cudaFree(p); p = nullptr; }
    for (double* p : {b.stage, b.tolWave, b.tolVortex, b.hostState}) if (p) cudaFree(p);
    if (b.errBits) cudaFree(b.errBits);
    if (b.errHost) cudaFreeHost(b.errHost);
    b.stage = b.tolWave = b.tolVortex = b.hostState = nullptr;
    b.errBits = nullptr;
    b.errHost = nullptr;
}

bool state_pointers_ok(const double* Ap, const double* Am, const double* A0) { return Ap && Am && A0; }

}  // namespace

extern "C" void wv_rk23_default_options(wv_rk23_options* o);

static int rk23_create_impl(wv_handle* handle, wv_system* system, const wv_rk23_options* options, wv_rk23** out) {
    if (!handle || !out) return WV_INVALID_POINTER;
    *out = nullptr;
    wv_rk23_options o;
    if (options) o = *options; else wv_rk23_default_options(&o);
    if (!wvgpu::rk23_options_valid(o)) return WV_INVALID_CONFIGURATION;
    if (!wvgpu::handle_is_single_state(handle)) return WV_UNSUPPORTED_OPERATION;
    const wvgpu::Descriptor& d = wvgpu::handle_descriptor(handle);
    std::vector<double> wave, vortex;
    const wvgpu::Status st = wvgpu::adaptive_error_tolerances(d, o.absolute_tolerance_scale, wave, vortex);
    if (!st) return st.code;
    auto* r = new (std::nothrow) wv_rk23(o);
    if (!r) return WV_ALLOCATION_FAILURE;
    // audit hash over every component's tolerances in layout order
    // (WVRungeKutta.cpp:602-613): A+, A-, A0, then each additional block's
    // uniform tolerance once per element
    r->hash = UINT64_C(1469598103934665603);
    for (int c = 0; c < 3; ++c) {
        r->componentHash[c] = UINT64_C(1469598103934665603);
        for (const double v : (c < 2 ? wave : vortex)) {
            r->hash = wvgpu::hash_tolerance(r->hash, v);
            r->componentHash[c] = wvgpu::hash_tolerance(r->componentHash[c], v);
        }
    }
    auto& b = r->backend;
    b.handle = handle;
    b.system = system;
    b.M = d.M;
    if (system) {
        std::vector<uint64_t> lengths;
        std::vector<double> tols;
        wvgpu::system_blocks(system, lengths, tols);
        for (size_t i = 0; i < lengths.size(); ++i)
            for (uint64_t j = 0; j < lengths[i]; ++j) r->hash = wvgpu::hash_tolerance(r->hash, tols[i]);
        b.nExtra = wvgpu::system_extra_doubles(system);
        b.tolExtra = wvgpu::system_extra_tolerances(system);
    }
    cudaSetDevice(wvgpu::handle_device(handle));
    const size_t sb = b.packed() * sizeof(double), tb = d.M * sizeof(double);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaMalloc(&b.k[i], sb);
    if (e == cudaSuccess) e = cudaMalloc(&b.stage, sb);
    if (e == cudaSuccess) e = cudaMalloc(&b.tolWave, tb);
    if (e == cudaSuccess) e = cudaMalloc(&b.tolVortex, tb);
    if (e == cudaSuccess) e = cudaMalloc(&b.errBits, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&b.errHost, sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(b.tolWave, wave.data(), tb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b.tolVortex, vortex.data(), tb, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        release(r);
        delete r;
        return e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_EXECUTION_FAILURE;
    }
    r->workspaceBytes = 5 * sb + 2 * tb;
    *out = r;
    return WV_SUCCESS;
}

extern "C" {

void wv_rk23_default_options(wv_rk23_options* o) {
    if (!o) return;
    o->relative_tolerance = 1e-3;
    o->absolute_tolerance_scale = 1e-6;
    o->safety_factor = 0.8;
    o->rejection_floor_factor = 0.5;
    o->maximum_step_factor = 5.0;
    o->maximum_step_size = std::numeric_limits<double>::infinity();
    o->maximum_recorded_step_diagnostics = 512;
}

int wv_rk23_create(wv_handle* handle, const wv_rk23_options* options, wv_rk23** out) {
    return rk23_create_impl(handle, nullptr, options, out);
}

int wv_rk23_create_for_system(wv_system* system, const wv_rk23_options* options, wv_rk23** out) {
    if (!system) return WV_INVALID_POINTER;
    return rk23_create_impl(wvgpu::system_handle(system), system, options, out);
}

void wv_rk23_destroy(wv_rk23* r) {
    if (!r) return;
    cudaSetDevice(wvgpu::handle_device(r->backend.handle));
    release(r);
    delete r;
}

const char* wv_rk23_last_message(const wv_rk23* r) { return r ? r->message.c_str() : "null integrator"; }

int wv_rk23_prepare_after_restart(wv_rk23* r) {
    if (!r) return WV_INVALID_POINTER;
    BusyGuard g(r->busy);
    if (!g.entered) return rk_fail(r, WV_REENTRANT_EXECUTION, "RK23 stepping is not reentrant.");
    r->controller.restart();
    return WV_SUCCESS;
}

static int rk23_run(wv_rk23* r, double* Ap, double* Am, double* A0, double* t, double t0, double a, double b, bool advance,
                    cudaStream_t s, double* packed = nullptr) {
    if (!std::isfinite(*t) || !std::isfinite(t0)) return rk_fail(r, WV_INVALID_CONFIGURATION, "State times must be finite.");
    BusyGuard g(r->busy);
    if (!g.entered) return rk_fail(r, WV_REENTRANT_EXECUTION, "RK23 stepping is not reentrant.");
    cudaSetDevice(wvgpu::handle_device(r->backend.handle));
    auto& be = r->backend;
    if (packed) be.bind_packed(be.base, packed);
    else be.base = {{Ap, Am, A0, nullptr}};
    be.t0 = t0;
    be.stream = s;
    double tt = *t;
    const int rc = advance ? r->controller.advance_to_time(tt, a, b) : r->controller.step(tt, a);
    if (rc) return rk_fail(r, rc, r->controller.message());
    *t = tt;
    return WV_SUCCESS;
}

int wv_rk23_step_device(wv_rk23* r, double* Ap, double* Am, double* A0, double* t, double t0, double proposed, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "A system integrator steps packed states (wv_rk23_system_*).");
    if (!state_pointers_ok(Ap, Am, A0) || !t) return rk_fail(r, WV_INVALID_POINTER, "RK23 received a null pointer.");
    return rk23_run(r, Ap, Am, A0, t, t0, proposed, 0.0, false, static_cast<cudaStream_t>(stream));
}

int wv_rk23_advance_to_time_device(wv_rk23* r, double* Ap, double* Am, double* A0, double* t, double t0, double final_time,
                                   double initial_step, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "A system integrator steps packed states (wv_rk23_system_*).");
    if (!state_pointers_ok(Ap, Am, A0) || !t) return rk_fail(r, WV_INVALID_POINTER, "RK23 received a null pointer.");
    return rk23_run(r, Ap, Am, A0, t, t0, final_time, initial_step, true, static_cast<cudaStream_t>(stream));
}

int wv_rk23_advance_to_time(wv_rk23* r, double* Ap, double* Am, double* A0, double* t, double t0, double final_time,
                            double initial_step) {
    if (!r) return WV_INVALID_POINTER;
    if (r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "A system integrator steps packed states (wv_rk23_system_*).");
    if (!state_pointers_ok(Ap, Am, A0) || !t) return rk_fail(r, WV_INVALID_POINTER, "RK23 received a null pointer.");
    auto& be = r->backend;
    cudaSetDevice(wvgpu::handle_device(be.handle));
    const size_t cb = 2 * be.M * sizeof(double);
    if (!be.hostState) {
        const cudaError_t e = cudaMalloc(&be.hostState, 3 * cb);
        if (e != cudaSuccess) return rk_fail(r, WV_ALLOCATION_FAILURE, "RK23 host-entry state allocation failed.");
        r->workspaceBytes += 3 * cb;
    }
    auto s = static_cast<cudaStream_t>(wvgpu::handle_stream(be.handle));
    double* host[] = {Ap, Am, A0};
    double* devs[] = {be.hostState, be.hostState + 2 * be.M, be.hostState + 4 * be.M};
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) e = cudaMemcpyAsync(devs[c], host[c], cb, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return rk_fail(r, WV_FFT_EXECUTION_FAILURE, std::string("RK23 state upload: ") + cudaGetErrorString(e));
    const int rc = rk23_run(r, devs[0], devs[1], devs[2], t, t0, final_time, initial_step, true, s);
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) e = cudaMemcpyAsync(host[c], devs[c], cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (rc) return rc;
    if (e != cudaSuccess) return rk_fail(r, WV_FFT_EXECUTION_FAILURE, std::string("RK23 state download: ") + cudaGetErrorString(e));
    return WV_SUCCESS;
}

int wv_rk23_dense_output_device(wv_rk23* r, double time, double* Ap, double* Am, double* A0, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "A system integrator steps packed states (wv_rk23_system_*).");
    if (!state_pointers_ok(Ap, Am, A0)) return rk_fail(r, WV_INVALID_POINTER, "Dense output received a null pointer.");
    BusyGuard g(r->busy);
    if (!g.entered) return rk_fail(r, WV_REENTRANT_EXECUTION, "RK23 dense-output evaluation is not reentrant.");
    cudaSetDevice(wvgpu::handle_device(r->backend.handle));
    auto& be = r->backend;
    be.denseOut = {{Ap, Am, A0, nullptr}};
    be.stream = static_cast<cudaStream_t>(stream);
    const int rc = r->controller.dense_output(time);
    if (rc) return rk_fail(r, rc, r->controller.message());
    return WV_SUCCESS;
}

int wv_rk23_system_step_device(wv_rk23* r, double* state, double* t, double t0, double proposed, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (!r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "The integrator is bound to a handle, not a system.");
    if (!state || !t) return rk_fail(r, WV_INVALID_POINTER, "RK23 received a null pointer.");
    return rk23_run(r, nullptr, nullptr, nullptr, t, t0, proposed, 0.0, false, static_cast<cudaStream_t>(stream), state);
}

int wv_rk23_system_advance_to_time_device(wv_rk23* r, double* state, double* t, double t0, double final_time,
                                          double initial_step, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (!r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "The integrator is bound to a handle, not a system.");
    if (!state || !t) return rk_fail(r, WV_INVALID_POINTER, "RK23 received a null pointer.");
    return rk23_run(r, nullptr, nullptr, nullptr, t, t0, final_time, initial_step, true, static_cast<cudaStream_t>(stream),
                    state);
}

int wv_rk23_system_dense_output_device(wv_rk23* r, double time, double* state, void* stream) {
    if (!r) return WV_INVALID_POINTER;
    if (!r->backend.system) return rk_fail(r, WV_UNSUPPORTED_OPERATION, "The integrator is bound to a handle, not a system.");
    if (!state) return rk_fail(r, WV_INVALID_POINTER, "Dense output received a null pointer.");
    BusyGuard g(r->busy);
    if (!g.entered) return rk_fail(r, WV_REENTRANT_EXECUTION, "RK23 dense-output evaluation is not reentrant.");
    cudaSetDevice(wvgpu::handle_device(r->backend.handle));
    auto& be = r->backend;
    be.bind_packed(be.denseOut, state);
    be.stream = static_cast<cudaStream_t>(stream);
    const int rc = r->controller.dense_output(time);
    if (rc) return rk_fail(r, rc, r->controller.message());
    return WV_SUCCESS;
}

int wv_rk23_next_step_size(const wv_rk23* r, double* next) {
    if (!r || !next) return WV_INVALID_POINTER;
    *next = r->controller.next_step_size();
    return WV_SUCCESS;
}

int wv_rk23_last_accepted_step(const wv_rk23* r, double* t_initial, double* t_final) {
    if (!r || !t_initial || !t_final) return WV_INVALID_POINTER;
    if (!r->controller.has_accepted_step()) return WV_UNSUPPORTED_OPERATION;
    *t_initial = r->controller.accepted_initial_time();
    *t_final = r->controller.accepted_final_time();
    return WV_SUCCESS;
}

int wv_rk23_get_metrics(const wv_rk23* r, wv_rk23_metrics* m) {
    if (!r || !m) return WV_INVALID_POINTER;
    *m = r->controller.metrics();
    m->workspace_bytes = r->workspaceBytes;
    return WV_SUCCESS;
}

int wv_rk23_get_diagnostics(const wv_rk23* r, wv_rk23_step_diagnostic* out, uint64_t capacity, uint64_t* count) {
    if (!r || !count) return WV_INVALID_POINTER;
    const auto& d = r->controller.diagnostics();
    *count = d.size();
    if (out)
        for (size_t i = 0; i < d.size() && i < capacity; ++i) out[i] = d[i];
    return WV_SUCCESS;
}

int wv_rk23_tolerance_hash(const wv_rk23* r, uint64_t* hash, uint64_t* component_hashes) {
    if (!r || !hash) return WV_INVALID_POINTER;
    *hash = r->hash;
    if (component_hashes)
        for (int c = 0; c < 3; ++c) component_hashes[c] = r->componentHash[c];
    return WV_SUCCESS;
}

}  // extern "C"

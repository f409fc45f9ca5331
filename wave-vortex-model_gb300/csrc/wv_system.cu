// Integration system with integrated observers (include/wvgpu.h, wv_system_*):
// WVConstantStratificationIntegrationSystem::evaluateRightHandSide
// (PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:295-400)
// on the device.  One scheduled flux per right-hand side also writes the
// advection fields (u, v, w); every tracer's F-grid advection and every
// particle group's velocity sampling reads those fields from HBM, so the
// shared "right-hand-side context" of the reference is one [3][Nx Ny Nz]
// buffer that never leaves the GPU.
//
// Particle velocities follow WVFieldEvaluationService::evaluateMovingImpl
// (PortableRuntime/src/WVFieldEvaluationService.cpp:1828-2030):
//   * linear: trilinear weights, periodic in x and y, clamped cell in z, the
//     eight products summed in the reference's loop order without contraction;
//   * spline: the not-a-knot cubic spline of each axis written as weights over
//     every grid point (SplineSystem, :116-259), x and y evaluated with the
//     query moved four cells away from a periodic seam and the weights rotated
//     back, then one contraction of the whole field with wx wy wz per particle.
// The spline weights are linear in the two nonzero entries of the spline's
// right-hand side, so each axis keeps a table q_k = D (A^T)^-1 e_k (A the
// not-a-knot system, D its second-difference read-out) built once on the host.
#include "wvgpu.h"
#include "wv_descriptor.hpp"
#include "wv_internal.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <new>
#include <string>
#include <vector>

namespace wvgpu {
namespace sysdev {

struct Grid {
    int Nx, Ny, Nz;
    double Lx, Ly, Lz, dx, dy, dz;
    size_t R;
};

// wrapped() of the field evaluation service: fmod into [0, L), L itself to 0.
__device__ __forceinline__ double wrapped(double c, double L) {
    double v = fmod(c, L);
    if (v < 0.0) v = __dadd_rn(v, L);
    if (v >= L) v = 0.0;
    return v;
}

// One thread per particle: (u, v[, w]) at the particle by trilinear interpolation.
__global__ void k_particles_linear(Grid g, const double* __restrict__ fields, const double* __restrict__ px,
                                   const double* __restrict__ py, const double* __restrict__ pz, int nch, size_t count,
                                   double* __restrict__ out0, double* __restrict__ out1, double* __restrict__ out2) {
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x) {
        const double x = wrapped(px[p], g.Lx), y = wrapped(py[p], g.Ly), z = pz[p];
        double val[3] = {0.0, 0.0, 0.0};
        if (z >= -g.Lz && z <= 0.0) {
            const size_t x0 = min(static_cast<size_t>(floor(x / g.dx)), static_cast<size_t>(g.Nx - 1));
            const size_t y0 = min(static_cast<size_t>(floor(y / g.dy)), static_cast<size_t>(g.Ny - 1));
            const double nz = __dadd_rn(z, g.Lz) / g.dz;
            const size_t z0 = min(static_cast<size_t>(fmax(0.0, floor(nz))), static_cast<size_t>(g.Nz - 2));
            const double wx1 = __dsub_rn(x, __dmul_rn(static_cast<double>(x0), g.dx)) / g.dx;
            const double wy1 = __dsub_rn(y, __dmul_rn(static_cast<double>(y0), g.dy)) / g.dy;
            const double wz1 = fmin(fmax(__dsub_rn(nz, static_cast<double>(z0)), 0.0), 1.0);
            const size_t xi[2] = {x0, (x0 + 1) % g.Nx}, yi[2] = {y0, (y0 + 1) % g.Ny};
            const double wx[2] = {__dsub_rn(1.0, wx1), wx1}, wy[2] = {__dsub_rn(1.0, wy1), wy1}, wz[2] = {__dsub_rn(1.0, wz1), wz1};
            const size_t plane = static_cast<size_t>(g.Nx) * g.Ny;
            for (int c = 0; c < nch; ++c) {
                const double* src = fields + c * g.R;
                double v = 0.0;
                for (int iz = 0; iz < 2; ++iz)
                    for (int iy = 0; iy < 2; ++iy)
                        for (int ix = 0; ix < 2; ++ix)
                            v = __dadd_rn(v, __dmul_rn(__dmul_rn(__dmul_rn(src[xi[ix] + g.Nx * yi[iy] + plane * (z0 + iz)], wx[ix]), wy[iy]),
                                                       wz[iz]));
                val[c] = v;
            }
        }
        out0[p] = val[0];
        out1[p] = val[1];
        if (nch > 2) out2[p] = val[2];
    }
}

// Spline weight of original grid index j on an axis of n points:
// SplineSystem::weightsInto with the circular shift folded in.
__device__ double spline_weight(int j, int n, double origin, double spacing, double query, int shift,
                                const double* __restrict__ q) {
    const double normalized = __dsub_rn(query, origin) / spacing;
    const int s = (j + shift) % n;  // index before restoreOriginalOrdering
    if (n == 2) return s == 0 ? __dsub_rn(1.0, normalized) : normalized;
    if (n == 3) {
        if (s == 0) return __dmul_rn(__dsub_rn(normalized, 1.0), __dsub_rn(normalized, 2.0)) / 2.0;
        if (s == 1) return __dmul_rn(-normalized, __dsub_rn(normalized, 2.0));
        return __dmul_rn(normalized, __dsub_rn(normalized, 1.0)) / 2.0;
    }
    int interval = normalized <= 0.0 ? 0 : static_cast<int>(floor(normalized));
    interval = min(interval, n - 2);
    const double fraction = fmin(fmax(__dsub_rn(normalized, static_cast<double>(interval)), 0.0), 1.0);
    const double first = __dsub_rn(1.0, fraction), second = fraction;
    const double a = __dsub_rn(__dmul_rn(__dmul_rn(first, first), first), first);
    const double b = __dsub_rn(__dmul_rn(__dmul_rn(second, second), second), second);
    double w = __dadd_rn(__dmul_rn(a, q[(size_t)interval * n + s]), __dmul_rn(b, q[(size_t)(interval + 1) * n + s]));
    if (s == interval) w = __dadd_rn(w, first);
    if (s == interval + 1) w = __dadd_rn(w, second);
    return w;
}

// One CTA per particle: the spline-interpolated (u, v[, w]) as the contraction
// of each whole field with wx wy wz.  Warps take (y, z) rows; lanes stride x.
__global__ void __launch_bounds__(256) k_particles_spline(Grid g, const double* __restrict__ fields, const double* __restrict__ px,
                                                         const double* __restrict__ py, const double* __restrict__ pz, int nch,
                                                         const double* __restrict__ qx, const double* __restrict__ qy,
                                                         const double* __restrict__ qz, double* __restrict__ out0,
                                                         double* __restrict__ out1, double* __restrict__ out2) {
    extern __shared__ __align__(16) double wsm[];
    double* wx = wsm;
    double* wy = wx + g.Nx;
    double* wz = wy + g.Ny;
    __shared__ double part[8][3];
    __shared__ int sValid;
    const size_t p = blockIdx.x;
    const double x = wrapped(px[p], g.Lx), y = wrapped(py[p], g.Ly), z = pz[p];
    const bool inside = z >= -g.Lz && z <= 0.0;
    const int xLower = static_cast<int>(min(static_cast<size_t>(floor(x / g.dx)), static_cast<size_t>(g.Nx - 1)));
    const int yLower = static_cast<int>(min(static_cast<size_t>(floor(y / g.dy)), static_cast<size_t>(g.Ny - 1)));
    const bool xBoundary = xLower < 3 || (g.Nx >= 4 && xLower > g.Nx - 4);
    const bool yBoundary = yLower < 3 || (g.Ny >= 4 && yLower > g.Ny - 4);
    const int xShift = xBoundary ? 4 : 0, yShift = yBoundary ? 4 : 0;
    const double xq = xBoundary ? wrapped(__dadd_rn(x, __dmul_rn(4.0, g.dx)), g.Lx) : x;
    const double yq = yBoundary ? wrapped(__dadd_rn(y, __dmul_rn(4.0, g.dy)), g.Ly) : y;
    const bool valid = inside && xq <= __dmul_rn(static_cast<double>(g.Nx - 1), g.dx) &&
                       yq <= __dmul_rn(static_cast<double>(g.Ny - 1), g.dy);
    if (threadIdx.x == 0) sValid = valid ? 1 : 0;
    for (int j = threadIdx.x; j < g.Nx; j += blockDim.x) wx[j] = spline_weight(j, g.Nx, 0.0, g.dx, xq, xShift % g.Nx, qx);
    for (int j = threadIdx.x; j < g.Ny; j += blockDim.x) wy[j] = spline_weight(j, g.Ny, 0.0, g.dy, yq, yShift % g.Ny, qy);
    for (int j = threadIdx.x; j < g.Nz; j += blockDim.x) wz[j] = spline_weight(j, g.Nz, -g.Lz, g.dz, z, 0, qz);
    __syncthreads();
    double acc[3] = {0.0, 0.0, 0.0};
    if (sValid) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        const int rows = g.Ny * g.Nz;
        for (int r = warp; r < rows; r += nw) {
            const int iy = r % g.Ny, iz = r / g.Ny;
            const size_t base = static_cast<size_t>(r) * g.Nx;
            double s[3] = {0.0, 0.0, 0.0};
            for (int ix = lane; ix < g.Nx; ix += 32)
                for (int c = 0; c < nch; ++c) s[c] = fma(fields[c * g.R + base + ix], wx[ix], s[c]);
            const double wyz = __dmul_rn(wy[iy], wz[iz]);
            for (int c = 0; c < nch; ++c) acc[c] = fma(s[c], wyz, acc[c]);
        }
        for (int c = 0; c < nch; ++c)
            for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], off);
        if (lane == 0)
            for (int c = 0; c < 3; ++c) part[warp][c] = acc[c];
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int c = 0; c < nch; ++c) {
                double v = 0.0;
                for (int w = 0; w < nw; ++w) v += part[w][c];
                acc[c] = v;
            }
        }
    }
    if (threadIdx.x == 0) {
        out0[p] = sValid ? acc[0] : 0.0;
        out1[p] = sValid ? acc[1] : 0.0;
        if (nch > 2) out2[p] = sValid ? acc[2] : 0.0;
    }
}

// RK4 stage arithmetic on packed states (IntegrationBuffer::setAffine / addScaled,
// PortableRuntime/src/WVRungeKutta.cpp:140-176), without contraction.
__global__ void k_sys_affine(const double* __restrict__ base, const double* __restrict__ inc, double scale,
                             double* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __dadd_rn(base[i], __dmul_rn(scale, inc[i]));
}
__global__ void k_sys_accumulate_and_stage(double* __restrict__ acc, const double* __restrict__ inc, double scale,
                                           const double* __restrict__ base, double cs, double* __restrict__ stage, int first,
                                           size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double k = inc[i];
        acc[i] = first ? k : __dadd_rn(acc[i], __dmul_rn(scale, k));
        if (stage) stage[i] = __dadd_rn(base[i], __dmul_rn(cs, k));
    }
}

}  // namespace sysdev

namespace {

// q tables of SplineSystem (WVFieldEvaluationService.cpp:116-259): A is the
// uniform-grid not-a-knot system (rows -1 2 -1 / 1 4 1 / -1 2 -1); the
// reference factors A^T with partial pivoting and reads shifted weights out
// of the solution c through the second difference at rows 1..n-2.  Row k of
// the table is that read-out for c = (A^T)^-1 e_k.
std::vector<double> spline_table(int n) {
    std::vector<double> q;
    if (n < 4) return q;
    std::vector<double> A(static_cast<size_t>(n) * n, 0.0);  // row-major A^T
    auto setA = [&](int row, int col, double v) { A[static_cast<size_t>(col) * n + row] = v; };
    setA(0, 0, -1.0); setA(0, 1, 2.0); setA(0, 2, -1.0);
    for (int r = 1; r + 1 < n; ++r) { setA(r, r - 1, 1.0); setA(r, r, 4.0); setA(r, r + 1, 1.0); }
    setA(n - 1, n - 3, -1.0); setA(n - 1, n - 2, 2.0); setA(n - 1, n - 1, -1.0);
    // LU with partial pivoting of A^T (Doolittle, in place)
    std::vector<int> piv(n);
    for (int c = 0; c < n; ++c) {
        int p = c;
        double best = std::abs(A[static_cast<size_t>(c) * n + c]);
        for (int r = c + 1; r < n; ++r)
            if (std::abs(A[static_cast<size_t>(r) * n + c]) > best) { best = std::abs(A[static_cast<size_t>(r) * n + c]); p = r; }
        piv[c] = p;
        if (p != c)
            for (int e = 0; e < n; ++e) std::swap(A[static_cast<size_t>(c) * n + e], A[static_cast<size_t>(p) * n + e]);
        for (int r = c + 1; r < n; ++r) {
            A[static_cast<size_t>(r) * n + c] /= A[static_cast<size_t>(c) * n + c];
            const double m = A[static_cast<size_t>(r) * n + c];
            for (int e = c + 1; e < n; ++e) A[static_cast<size_t>(r) * n + e] -= m * A[static_cast<size_t>(c) * n + e];
        }
    }
    q.assign(static_cast<size_t>(n) * n, 0.0);
    std::vector<double> rhs(n);
    for (int k = 0; k < n; ++k) {
        std::fill(rhs.begin(), rhs.end(), 0.0);
        rhs[k] = 1.0;
        for (int c = 0; c < n; ++c) {
            if (piv[c] != c) std::swap(rhs[c], rhs[piv[c]]);
            for (int r = c + 1; r < n; ++r) rhs[r] -= A[static_cast<size_t>(r) * n + c] * rhs[c];
        }
        for (int r = n - 1; r >= 0; --r) {
            for (int c = r + 1; c < n; ++c) rhs[r] -= A[static_cast<size_t>(r) * n + c] * rhs[c];
            rhs[r] /= A[static_cast<size_t>(r) * n + r];
        }
        double* row = q.data() + static_cast<size_t>(k) * n;
        for (int r = 1; r + 1 < n; ++r) {
            row[r - 1] += rhs[r];
            row[r] -= 2.0 * rhs[r];
            row[r + 1] += rhs[r];
        }
    }
    return q;
}

}  // namespace
}  // namespace wvgpu

struct wv_system {
    struct Group {
        size_t count = 0, xOff = 0, yOff = 0, zOff = 0, zFixedOff = 0;
        bool xyOnly = false;
        int interpolation = WV_INTERPOLATION_LINEAR;
    };
    struct Tracer {
        size_t off = 0;
        bool antialias = true;
    };
    wv_handle* h = nullptr;
    size_t M = 0, R = 0, nExtra = 0, nState = 0;
    wvgpu::sysdev::Grid grid{};
    std::vector<Group> groups;
    std::vector<Tracer> tracers;
    std::vector<uint64_t> blockOffset, blockLength;
    std::vector<double> blockTolerance;
    double* fields = nullptr;   // [3][R]
    double* zFixed = nullptr;   // depths of xy-only particles
    double* q[3] = {};          // spline tables of x, y, z
    double* tolExtra = nullptr; // [nExtra]
    double* acc = nullptr;      // RK4 workspace, packed state each
    double* stage = nullptr;
    double* kbuf = nullptr;
    double* hostMirror = nullptr;
    bool hasSpline = false;
    std::string message;
    std::atomic<bool> busy{false};
};

namespace {

int sys_fail(wv_system* s, int code, const std::string& m) {
    if (s) s->message = m;
    return code;
}

int sys_cuda(wv_system* s, cudaError_t e, const char* where) {
    if (e == cudaSuccess) return WV_SUCCESS;
    return sys_fail(s, e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_EXECUTION_FAILURE,
                    std::string(where) + ": " + cudaGetErrorString(e));
}

struct SysGuard {
    std::atomic<bool>& flag;
    bool entered;
    explicit SysGuard(std::atomic<bool>& f) : flag(f), entered(!f.exchange(true)) {}
    ~SysGuard() { if (entered) flag.store(false); }
};

void release(wv_system* s) {
    for (double* p : {s->fields, s->zFixed, s->q[0], s->q[1], s->q[2], s->tolExtra, s->acc, s->stage, s->kbuf, s->hostMirror})
        if (p) cudaFree(p);
}

unsigned grid_for(size_t n) { return static_cast<unsigned>(std::min<size_t>((n + 255) / 256, wvgpu::grid_cap(8))); }

// evaluateRightHandSide on packed device arrays (no guard; callers hold it).
int rhs_impl(wv_system* s, double t, double t0, const double* x, double* k, cudaStream_t st) {
    const size_t M2 = 2 * s->M;
    int rc = wvgpu::scheduled_rhs_with_fields(s->h, t, t0, x, x + M2, x + 2 * M2, k, k + M2, k + 2 * M2, s->fields, st);
    if (rc) return sys_fail(s, rc, wv_last_message(s->h));
    const double* xe = x + 6 * s->M;
    double* ke = k + 6 * s->M;
    for (const auto& tr : s->tracers) {
        rc = wv_advect_fgrid_scalar_device(s->h, xe + tr.off, s->fields, tr.antialias ? 1 : 0, ke + tr.off, st);
        if (rc) return sys_fail(s, rc, wv_last_message(s->h));
    }
    const auto& g = s->grid;
    for (const auto& gr : s->groups) {
        if (gr.count == 0) continue;
        const double* pz = gr.xyOnly ? s->zFixed + gr.zFixedOff : xe + gr.zOff;
        const int nch = gr.xyOnly ? 2 : 3;
        double* o2 = gr.xyOnly ? nullptr : ke + gr.zOff;
        if (gr.interpolation == WV_INTERPOLATION_SPLINE) {
            const size_t smem = static_cast<size_t>(g.Nx + g.Ny + g.Nz) * sizeof(double);
            wvgpu::sysdev::k_particles_spline<<<static_cast<unsigned>(gr.count), 256, smem, st>>>(
                g, s->fields, xe + gr.xOff, xe + gr.yOff, pz, nch, s->q[0], s->q[1], s->q[2], ke + gr.xOff, ke + gr.yOff, o2);
        } else {
            wvgpu::sysdev::k_particles_linear<<<grid_for(gr.count), 256, 0, st>>>(g, s->fields, xe + gr.xOff, xe + gr.yOff, pz, nch,
                                                                                 gr.count, ke + gr.xOff, ke + gr.yOff, o2);
        }
        rc = sys_cuda(s, cudaGetLastError(), "particle velocities");
        if (rc) return rc;
    }
    return WV_SUCCESS;
}

// WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462) on the
// packed state y (in place).
int rk4_step(wv_system* s, double* y, double t, double t0, double dt, cudaStream_t st) {
    using namespace wvgpu::sysdev;
    const size_t n = s->nState;
    const unsigned gr = grid_for(n);
    int rc = rhs_impl(s, t, t0, y, s->kbuf, st); if (rc) return rc;
    k_sys_accumulate_and_stage<<<gr, 256, 0, st>>>(s->acc, s->kbuf, 1.0, y, 0.5 * dt, s->stage, 1, n);
    rc = rhs_impl(s, t + 0.5 * dt, t0, s->stage, s->kbuf, st); if (rc) return rc;
    k_sys_accumulate_and_stage<<<gr, 256, 0, st>>>(s->acc, s->kbuf, 2.0, y, 0.5 * dt, s->stage, 0, n);
    rc = rhs_impl(s, t + 0.5 * dt, t0, s->stage, s->kbuf, st); if (rc) return rc;
    k_sys_accumulate_and_stage<<<gr, 256, 0, st>>>(s->acc, s->kbuf, 2.0, y, dt, s->stage, 0, n);
    rc = rhs_impl(s, t + dt, t0, s->stage, s->kbuf, st); if (rc) return rc;
    k_sys_accumulate_and_stage<<<gr, 256, 0, st>>>(s->acc, s->kbuf, 1.0, nullptr, 0.0, nullptr, 0, n);
    k_sys_affine<<<gr, 256, 0, st>>>(y, s->acc, dt / 6.0, y, n);
    return sys_cuda(s, cudaGetLastError(), "RK4 stage arithmetic");
}

}  // namespace

namespace wvgpu {
int system_rhs(wv_system* s, double t, double t0, const double* state, double* rhs, void* stream) {
    return rhs_impl(s, t, t0, state, rhs, static_cast<cudaStream_t>(stream));
}
size_t system_extra_doubles(const wv_system* s) { return s->nExtra; }
const double* system_extra_tolerances(const wv_system* s) { return s->tolExtra; }
wv_handle* system_handle(const wv_system* s) { return s->h; }
void system_blocks(const wv_system* s, std::vector<uint64_t>& lengths, std::vector<double>& tolerances) {
    lengths = s->blockLength;
    tolerances = s->blockTolerance;
}
}  // namespace wvgpu

extern "C" {

int wv_system_create(wv_handle* h, const wv_particle_group* groups, int n_groups, const wv_tracer* tracers, int n_tracers,
                     wv_system** out) {
    if (!h || !out) return WV_INVALID_POINTER;
    *out = nullptr;
    if (n_groups < 0 || n_tracers < 0 || (n_groups > 0 && !groups) || (n_tracers > 0 && !tracers)) return WV_INVALID_POINTER;
    if (!wvgpu::handle_is_single_state(h)) return WV_UNSUPPORTED_OPERATION;
    const wvgpu::Descriptor& d = wvgpu::handle_descriptor(h);
    auto* s = new (std::nothrow) wv_system;
    if (!s) return WV_ALLOCATION_FAILURE;
    s->h = h;
    s->M = d.M;
    const size_t Nx = d.c.Nx, Ny = d.c.Ny, Nz = d.c.Nz;
    s->R = Nx * Ny * Nz;
    s->grid = {static_cast<int>(Nx), static_cast<int>(Ny), static_cast<int>(Nz), d.c.Lx, d.c.Ly, d.c.Lz,
               d.c.Lx / static_cast<double>(Nx), d.c.Ly / static_cast<double>(Ny), d.c.Lz / static_cast<double>(Nz - 1), s->R};
    std::vector<double> zf, tol;
    size_t off = 0;
    auto addBlock = [&](size_t len, double t) {
        s->blockOffset.push_back(6 * d.M + off);
        s->blockLength.push_back(len);
        s->blockTolerance.push_back(t);
        tol.insert(tol.end(), len, t);
        off += len;
        return off - len;
    };
    for (int gi = 0; gi < n_groups; ++gi) {
        const auto& g = groups[gi];
        wv_system::Group gr;
        gr.count = g.count;
        gr.xyOnly = g.xy_only != 0;
        gr.interpolation = g.interpolation;
        if (g.interpolation != WV_INTERPOLATION_LINEAR && g.interpolation != WV_INTERPOLATION_SPLINE) {
            delete s;
            return WV_INVALID_CONFIGURATION;
        }
        if (gr.xyOnly && g.count > 0 && !g.z_fixed) {
            delete s;
            return WV_INVALID_POINTER;  // xy particles need one fixed depth per particle
        }
        gr.xOff = addBlock(g.count, g.horizontal_tolerance);
        gr.yOff = addBlock(g.count, g.horizontal_tolerance);
        if (!gr.xyOnly) gr.zOff = addBlock(g.count, g.vertical_tolerance);
        else {
            gr.zFixedOff = zf.size();
            zf.insert(zf.end(), g.z_fixed, g.z_fixed + g.count);
        }
        if (g.interpolation == WV_INTERPOLATION_SPLINE && g.count > 0) s->hasSpline = true;
        s->groups.push_back(gr);
    }
    for (int i = 0; i < n_tracers; ++i) {
        wv_system::Tracer tr;
        tr.antialias = tracers[i].antialias != 0;
        tr.off = addBlock(s->R, tracers[i].absolute_tolerance);
        s->tracers.push_back(tr);
    }
    s->nExtra = off;
    s->nState = 6 * d.M + off;
    cudaSetDevice(wvgpu::handle_device(h));
    const size_t sb = s->nState * sizeof(double);
    cudaError_t e = cudaMalloc(&s->fields, 3 * s->R * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->acc, sb);
    if (e == cudaSuccess) e = cudaMalloc(&s->stage, sb);
    if (e == cudaSuccess) e = cudaMalloc(&s->kbuf, sb);
    if (e == cudaSuccess && !zf.empty()) e = cudaMalloc(&s->zFixed, zf.size() * sizeof(double));
    if (e == cudaSuccess && !zf.empty()) e = cudaMemcpy(s->zFixed, zf.data(), zf.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && off > 0) e = cudaMalloc(&s->tolExtra, off * sizeof(double));
    if (e == cudaSuccess && off > 0) e = cudaMemcpy(s->tolExtra, tol.data(), off * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && s->hasSpline) {
        const size_t n[3] = {Nx, Ny, Nz};
        for (int a = 0; a < 3 && e == cudaSuccess; ++a) {
            const auto tab = wvgpu::spline_table(static_cast<int>(n[a]));
            if (tab.empty()) continue;
            e = cudaMalloc(&s->q[a], tab.size() * sizeof(double));
            if (e == cudaSuccess) e = cudaMemcpy(s->q[a], tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice);
        }
    }
    if (e == cudaSuccess && s->hasSpline) {
        const size_t smem = (Nx + Ny + Nz) * sizeof(double);
        if (smem > 48 * 1024)
            e = cudaFuncSetAttribute(wvgpu::sysdev::k_particles_spline, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem));
    }
    if (e != cudaSuccess) {
        release(s);
        delete s;
        return e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_EXECUTION_FAILURE;
    }
    *out = s;
    return WV_SUCCESS;
}

void wv_system_destroy(wv_system* s) {
    if (!s) return;
    cudaSetDevice(wvgpu::handle_device(s->h));
    release(s);
    delete s;
}

const char* wv_system_last_message(const wv_system* s) { return s ? s->message.c_str() : "null system"; }

int wv_system_get_layout(const wv_system* s, uint64_t* state_doubles, uint64_t* n_blocks, uint64_t* offsets,
                         uint64_t* lengths, uint64_t capacity) {
    if (!s) return WV_INVALID_POINTER;
    if (state_doubles) *state_doubles = s->nState;
    if (n_blocks) *n_blocks = s->blockOffset.size();
    for (size_t i = 0; i < s->blockOffset.size() && i < capacity; ++i) {
        if (offsets) offsets[i] = s->blockOffset[i];
        if (lengths) lengths[i] = s->blockLength[i];
    }
    return WV_SUCCESS;
}

int wv_system_rhs_device(wv_system* s, double t, double t0, const double* state, double* rhs, void* stream) {
    if (!s) return WV_INVALID_POINTER;
    if (!state || !rhs) return sys_fail(s, WV_INVALID_POINTER, "Integration RHS received a null pointer.");
    SysGuard g(s->busy);
    if (!g.entered) return sys_fail(s, WV_REENTRANT_EXECUTION, "The constant-stratification integration system is not reentrant.");
    cudaSetDevice(wvgpu::handle_device(s->h));
    return rhs_impl(s, t, t0, state, rhs, static_cast<cudaStream_t>(stream));
}

int wv_system_rk4_device(wv_system* s, double* state, double* t, double t0, double dt, int n, void* stream) {
    if (!s) return WV_INVALID_POINTER;
    if (!state || !t) return sys_fail(s, WV_INVALID_POINTER, "RK4 received a null pointer.");
    if (!std::isfinite(*t) || !std::isfinite(t0)) return sys_fail(s, WV_INVALID_CONFIGURATION, "State times must be finite.");
    if (!(dt > 0.0) || !std::isfinite(dt)) return sys_fail(s, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    if (n < 0) return sys_fail(s, WV_INVALID_CONFIGURATION, "RK4 step count must be nonnegative.");
    SysGuard g(s->busy);
    if (!g.entered) return sys_fail(s, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    cudaSetDevice(wvgpu::handle_device(s->h));
    auto st = static_cast<cudaStream_t>(stream);
    double tt = *t;
    for (int i = 0; i < n; ++i) {
        const int rc = rk4_step(s, state, tt, t0, dt, st);
        if (rc) return rc;
        tt = tt + dt;
    }
    *t = tt;
    return WV_SUCCESS;
}

int wv_system_rk4(wv_system* s, double* state, double* t, double t0, double dt, int n) {
    if (!s) return WV_INVALID_POINTER;
    if (!state || !t) return sys_fail(s, WV_INVALID_POINTER, "RK4 received a null pointer.");
    cudaSetDevice(wvgpu::handle_device(s->h));
    const size_t bytes = s->nState * sizeof(double);
    if (!s->hostMirror) {
        const cudaError_t e = cudaMalloc(&s->hostMirror, bytes);
        if (e != cudaSuccess) return sys_fail(s, WV_ALLOCATION_FAILURE, "Integration state mirror allocation failed.");
    }
    auto st = static_cast<cudaStream_t>(wvgpu::handle_stream(s->h));
    cudaError_t e = cudaMemcpyAsync(s->hostMirror, state, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return sys_cuda(s, e, "state upload");
    const int rc = wv_system_rk4_device(s, s->hostMirror, t, t0, dt, n, st);
    e = cudaMemcpyAsync(state, s->hostMirror, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (rc) return rc;
    return sys_cuda(s, e, "state download");
}

}  // extern "C"

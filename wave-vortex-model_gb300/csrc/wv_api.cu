// C ABI of the GB300 constant-stratification spectral step (include/wvgpu.h).
//
// A handle owns: the FP64 descriptor and layout plan (built on the host,
// uploaded once), the device scratch arena of the flux pipeline, device
// mirrors for the host-pointer entry points and the RK4 workspace.  Caller
// buffers are never retained.  Calls on one handle are not reentrant
// (ExecutionGuard, CompiledKernel/src/WVTransformConstantStratificationKernel.cpp:76-84).
#include "wvgpu.h"
#include "wv_descriptor.hpp"
#include "wv_internal.hpp"
#include "wv_kernels.cuh"
#include "wv_plan.hpp"
#include "wv_warpfft.cuh"
#include "wv_adjoint.cuh"
#include "wv_vinv_tc.cuh"
#include "wv_vfwd_tc.cuh"
#include "wv_vinv_tcx.cuh"
#include "wv_vfft.cuh"
#include "wv_scalar.cuh"

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <cmath>
#include <limits>
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include <type_traits>

using wvgpu::Descriptor;
using wvgpu::Plan;
using wvgpu::Status;
namespace dev = wvgpu::dev;

struct wv_handle {
    Descriptor desc;
    Plan plan;
    int precision = WV_PRECISION_FP64;
    uint32_t forcing = WV_FORCING_NONLINEAR_ADVECTION;
    std::string message;
    std::atomic<bool> busy{false};
    wv_metrics metrics{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocations;
    size_t deviceBytes = 0;
    dev::DescDev dd{};
    // pipeline scratch (typed by precision)
    void* zspec = nullptr;
    void* yspec = nullptr;
    void* pspec = nullptr;
    void* fspec = nullptr;
    unsigned long long* maxSpeed = nullptr;
    // host-entry mirrors and RK4 workspace, [3][M] complex each
    double* state = nullptr;
    double* flux = nullptr;
    double* stage = nullptr;
    double* kbuf = nullptr;
    double* acc = nullptr;
    double* fields = nullptr;  // [4][R] doubles
    bool hasDamping = false;
    // adjoint workspace (allocated on the first adjoint call)
    bool adjointReady = false;
    void* zadj = nullptr;   // [nt][z][pos]
    void* yadj = nullptr;   // [z][nt][y][kx]
    void* yout = nullptr;   // [z][4+2nt][y][kx]
    void* fadj = nullptr;   // [4+2nt][z][pos]
    double* st[4] = {};     // RK4 stage states (st[1..3]) for the step adjoint
    double* kb = nullptr;
    double* sb = nullptr;
    double* ybacc = nullptr;
    double* ybin = nullptr;
    std::vector<double*> checkpoints;  // multi-step adjoint: saved states
    std::vector<double*> segment;      // multi-step adjoint: states of one segment
    std::vector<void*> ystore;         // multi-step adjoint: x-pass real rows of each stage flux of one segment
    cudaStream_t adjStream = nullptr;  // multi-step adjoint: recomputation of the next segment
    double* ybAlt = nullptr;           // multi-step adjoint: second cotangent buffer
    cudaEvent_t slotReady[2] = {}, slotFree[2] = {}, fwdDone = nullptr;
    // RK4 dense output (WVFixedStepRK4Options::retainDenseOutput): state before
    // and after the last step, its first and fourth stage derivatives, [4][3][M]
    bool rk4Dense = false;
    double* denseBuf = nullptr;
    bool denseValid = false;
    double denseTi = 0.0, denseTf = 0.0;
    bool instrument = false;
    bool tcAvailable = false;  // tensor-core vertical inverse transform built for this handle
    // kernels of the flux's vertical inverse and forward transforms (WV_VERTICAL_*)
    int vinvKind = WV_VERTICAL_CUDA_CORES;
    int vfwdKind = WV_VERTICAL_CUDA_CORES;
    size_t tcSmem = 0;
    bool tcFwdAvailable = false;  // tensor-core forward vertical transform built (mixed handles)
    size_t tcFwdSmem = 0;
    size_t tcxSmem = 0;           // FP32X2: shared memory of the digit-sliced tensor-core inverse
    // F-grid scalar advection (built on first use): full-spectrum descriptor copy,
    // z-derivative matrix, per-position flags and scratch
    bool scalarReady = false;
    dev::DescDev sd{};
    const void* scalarD = nullptr;
    const unsigned char* scalarFlags = nullptr;
    void* scalarP = nullptr;      // [z][3][y][NxHalf] complex (x r2c / y inverse side)
    void* scalarF = nullptr;      // [4][z][pos] complex (y forward side)
    double* scalarGrad = nullptr; // [3][R] doubles
    double* scalarRhs = nullptr;  // [R] doubles (host-pointer entry)
    cudaEvent_t ev[6] = {};
    wv_stage_times stages{};
    // test hooks (wv_test_*): flux launch sequences to let through before one
    // fails (-1: off), and whether the last failure was the injected one
    long long failLaunchAfter = -1;
    bool injectedFailure = false;
};

namespace {

// Test hooks: device allocations of the handles to let through before one
// fails (-1: off), and the device bytes the handles hold right now.
std::atomic<long long> g_failAllocationAfter{-1};
std::atomic<long long> g_liveDeviceBytes{0};

bool injected_allocation_failure() {
    if (g_failAllocationAfter.load() < 0) return false;
    return g_failAllocationAfter.fetch_sub(1) == 0;
}

struct Guard {
    std::atomic<bool>& flag;
    bool entered;
    explicit Guard(std::atomic<bool>& f) : flag(f), entered(!f.exchange(true)) {}
    ~Guard() { if (entered) flag.store(false); }
};

int fail(wv_handle* h, int code, const std::string& message) {
    if (h) h->message = message;
    return code;
}

int cuda_fail(wv_handle* h, cudaError_t e, const char* where) {
    const int code = e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_EXECUTION_FAILURE;
    if (h && h->injectedFailure) {
        h->injectedFailure = false;
        return fail(h, code, std::string(where) + ": injected execution failure");
    }
    return fail(h, code, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename V>
cudaError_t upload(wv_handle* h, const std::vector<V>& host, const V** out) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(host.size() * sizeof(V), 16);
    if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return e;
    h->allocations.push_back(p);
    h->deviceBytes += bytes;
    g_liveDeviceBytes += static_cast<long long>(bytes);
    if (!host.empty()) e = cudaMemcpy(p, host.data(), host.size() * sizeof(V), cudaMemcpyHostToDevice);
    *out = static_cast<const V*>(p);
    return e;
}

cudaError_t alloc(wv_handle* h, size_t bytes, void** out) {
    void* p = nullptr;
    bytes = std::max<size_t>(bytes, 16);
    if (injected_allocation_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) return e;
    h->allocations.push_back(p);
    h->deviceBytes += bytes;
    g_liveDeviceBytes += static_cast<long long>(bytes);
    *out = p;
    return cudaMemset(p, 0, bytes);
}

std::vector<double> interleave(const std::vector<wvgpu::cdouble>& v) {
    std::vector<double> out(2 * v.size());
    for (size_t i = 0; i < v.size(); ++i) { out[2 * i] = v[i].real(); out[2 * i + 1] = v[i].imag(); }
    return out;
}

template <typename T>
std::vector<T> cast(const std::vector<double>& v) { return std::vector<T>(v.begin(), v.end()); }

// BF16 with round-to-nearest-even from an FP32 value (host), and back.
uint16_t bf16_rne(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}
double bf16_value(uint16_t h) {
    const uint32_t u = static_cast<uint32_t>(h) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// The folded inverse matrices Ccos, Csin, CcosM, CsinM ([zHalf][Nj], FP64) as
// three BF16 pieces each (hi, the rounded remainder, the rounded remainder of
// that), laid out for the tensor-core vertical transform: row n < NP, column
// kk < K with even j = 2 kk in kk < KE and odd j = 2 (kk - KE) + 1 after it,
// canonical no-swizzle K-major core matrices; zeros outside the matrix.
std::vector<uint16_t> tc_vertical_blob(const Plan& p, int NP, int KE, int K) {
    const size_t split = static_cast<size_t>(NP) * K;  // BF16 entries per piece
    std::vector<uint16_t> out(4 * 3 * split, 0);
    const std::vector<double>* mats[4] = {&p.Ccos, &p.Csin, &p.CcosM, &p.CsinM};
    const int Zh = static_cast<int>(p.zHalf), Nj = static_cast<int>(p.Nj);
    for (int m = 0; m < 4; ++m)
        for (int n = 0; n < Zh; ++n)
            for (int kk = 0; kk < K; ++kk) {
                const int j = kk < KE ? 2 * kk : 2 * (kk - KE) + 1;
                if (j >= Nj || (kk >= KE && kk - KE >= (Nj / 2))) continue;
                if (kk < KE && kk >= (Nj + 1) / 2) continue;
                const double c = (*mats[m])[static_cast<size_t>(n) * Nj + j];
                const uint16_t hb = bf16_rne(static_cast<float>(c));
                const double r1 = c - bf16_value(hb);
                const uint16_t mb = bf16_rne(static_cast<float>(r1));
                const double r2 = r1 - bf16_value(mb);
                const uint16_t lb = bf16_rne(static_cast<float>(r2));
                const size_t e = dev::tc_kmajor_offset(n, kk, K) / 2;
                out[(static_cast<size_t>(m) * 3 + 0) * split + e] = hb;
                out[(static_cast<size_t>(m) * 3 + 1) * split + e] = mb;
                out[(static_cast<size_t>(m) * 3 + 2) * split + e] = lb;
            }
    return out;
}

// The forward matrices Fcos, Fsin ([Nj][zHalf], FP64) as three BF16 pieces,
// laid out for the tensor-core forward transform: [family cos|sin][parity
// even|odd][piece][NF rows][KF], row c holding output j = 2 c + parity, column
// k = n < zHalf, canonical no-swizzle K-major core matrices; zeros elsewhere.
std::vector<uint16_t> tc_forward_blob(const Plan& p, int NF, int KF) {
    const size_t split = static_cast<size_t>(NF) * KF;
    std::vector<uint16_t> out(2 * 2 * 3 * split, 0);
    const std::vector<double>* mats[2] = {&p.Fcos, &p.Fsin};
    const int Zh = static_cast<int>(p.zHalf), Nj = static_cast<int>(p.Nj);
    for (int m = 0; m < 2; ++m)
        for (int j = 0; j < Nj; ++j)
            for (int n = 0; n < Zh; ++n) {
                const double c = (*mats[m])[static_cast<size_t>(j) * Zh + n];
                const uint16_t hb = bf16_rne(static_cast<float>(c));
                const double r1 = c - bf16_value(hb);
                const uint16_t mb = bf16_rne(static_cast<float>(r1));
                const double r2 = r1 - bf16_value(mb);
                const uint16_t lb = bf16_rne(static_cast<float>(r2));
                const size_t e = dev::tc_kmajor_offset(j >> 1, n, KF) / 2;
                const size_t blk = static_cast<size_t>(m) * 2 + (j & 1);
                out[(blk * 3 + 0) * split + e] = hb;
                out[(blk * 3 + 1) * split + e] = mb;
                out[(blk * 3 + 2) * split + e] = lb;
            }
    return out;
}

// The inverse matrices Ccos, Csin, Ccos, -Csin (the z-derivative matrices
// m_j Ccos and -m_j Csin with m_j moved into the A operand) as six balanced
// base-256 digit slices per row for the FP32X2 tensor-core inverse
// (k_vinv_tcx): row n of matrix m is scaled by 2^-F (F = tcxF[m][n], the
// smallest F with max_j |C[n][j]| < 2^F), rounded to the integer
// Y = round(C 2^(47-F)) and written as digits D_0 .. D_5 (Y = sum_s D_s
// 256^(5-s), D_s in [-128, 128]); slice s holds the BF16 value D_s 2^(-7-8s)
// (exact).  Blocks [matrix][j parity][pass][slice][NP rows][KH] (output row
// n = pass NP + row; even j = 2 k in parity 0, odd j = 2 k + 1 in parity 1),
// canonical no-swizzle K-major layout; zeros outside the matrix.
struct DigitBlob {
    std::vector<uint16_t> blob;
    std::vector<int32_t> F;
};
DigitBlob tc_digit_blob(const Plan& p, int NP, int KH, int passes) {
    const size_t split = static_cast<size_t>(NP) * KH;
    const size_t rows = static_cast<size_t>(NP) * passes;
    DigitBlob out;
    out.blob.assign(4 * 2 * rows * dev::kTcxDigits * KH, 0);
    out.F.assign(4 * rows, 0);
    const std::vector<double>* mats[4] = {&p.Ccos, &p.Csin, &p.Ccos, &p.Csin};
    const double sign[4] = {1.0, 1.0, 1.0, -1.0};
    const int Zh = static_cast<int>(p.zHalf), Nj = static_cast<int>(p.Nj);
    for (int m = 0; m < 4; ++m)
        for (int n = 0; n < Zh; ++n) {
            const double* row = mats[m]->data() + static_cast<size_t>(n) * Nj;
            double mx = 0.0;
            for (int j = 0; j < Nj; ++j) mx = std::max(mx, std::fabs(row[j]));
            int F = 0;
            if (mx > 0.0) std::frexp(mx, &F);
            out.F[static_cast<size_t>(m) * rows + n] = F;
            const int pass = n / NP, rn = n % NP;
            for (int j = 0; j < Nj; ++j) {
                long long Y = std::llround(std::ldexp(sign[m] * row[j], 47 - F));
                int D[dev::kTcxDigits];
                for (int s2 = dev::kTcxDigits - 1; s2 >= 1; --s2) {
                    int dd = static_cast<int>(Y & 0xFFll);
                    dd -= (dd & 0x80) << 1;
                    D[s2] = dd;
                    Y = (Y - dd) / 256;
                }
                D[0] = static_cast<int>(Y);
                const size_t e = dev::tc_kmajor_offset(rn, j >> 1, KH) / 2;
                const size_t blk = (static_cast<size_t>(m) * 2 + (j & 1)) * passes + pass;
                for (int s2 = 0; s2 < dev::kTcxDigits; ++s2)
                    out.blob[(blk * dev::kTcxDigits + s2) * split + e] =
                        bf16_rne(static_cast<float>(std::ldexp(static_cast<double>(D[s2]), -7 - 8 * s2)));
            }
        }
    return out;
}

// Flux projection of the mixed form, folded per (mode, j) in FP64 and rounded
// once to FP32 (projectFluxTargetMode, kernel.cpp:396-431, written as one
// linear map of the channel values u, v, w, eta):
//   f0   = i Du u + i Dv v + Dn eta
//   wave = Cu u + Cv v + Cw w,   b = Npm eta - B f0,   cp = wave + b,  cm = wave - b
// Layout [M][12]: Cu.re Cu.im Cv.re Cv.im | Cw.re Cw.im Du Dv | Dn Npm B 0.
// The inertial row (mode 0) keeps its own formula in the kernel.
std::vector<double> mixed_flux_projection(const wvgpu::Descriptor& d) {
    std::vector<double> out(12 * d.M, 0.0);
    const bool hydro = d.c.is_hydrostatic;
    const size_t Nj = d.c.Nj;
    for (size_t w = 0; w < d.Nkl; ++w) {
        for (size_t j = 0; j < Nj; ++j) {
            const size_t idx = j + Nj * w;
            double* o = out.data() + 12 * idx;
            double cu[2] = {0, 0}, cv[2] = {0, 0}, cw[2] = {0, 0};
            if (hydro) {
                const double ar = d.ApmD[idx].real(), ai = d.ApmD[idx].imag();
                cu[0] = -d.k[w] * ai; cu[1] = d.k[w] * ar;   // i k ApmD
                cv[0] = -d.l[w] * ai; cv[1] = d.l[w] * ar;   // i l ApmD
            } else {
                cu[0] = d.cosAlpha[w] * d.ApmDScaled[idx];
                cv[0] = d.sinAlpha[w] * d.ApmDScaled[idx];
                cw[1] = (d.Kh[w] / 2.0) * d.apmWProjectionPrefactor[j];
            }
            o[0] = cu[0]; o[1] = cu[1]; o[2] = cv[0]; o[3] = cv[1];
            o[4] = cw[0]; o[5] = cw[1];
            o[6] = -d.l[w] * d.A0FromVorticity[idx];
            o[7] = d.k[w] * d.A0FromVorticity[idx];
            o[8] = d.A0FromBuoyancy[idx];
            o[9] = d.ApmN[idx];
            o[10] = d.NA0[idx] * d.ApmN[idx];
        }
    }
    return out;
}

size_t elem_size(int precision) {
    return precision == WV_PRECISION_FP64 ? sizeof(double) : precision == WV_PRECISION_MIXED ? sizeof(float) : sizeof(dev::ff);
}

// Scratch element counts (complex) of the flux pipeline.
struct ScratchSizes { size_t z, y, p, f; };
ScratchSizes scratch_sizes(const Plan& p) {
    const size_t nt = p.targets.count;
    ScratchSizes s;
    s.z = (4 + nt) * p.Nz * p.positions;
    s.y = p.Nz * (4 + 2 * nt) * p.Ny * p.kxColumns;
    s.p = p.Nz * 4 * p.Ny * p.kxColumns;
    s.f = 4 * p.Nz * p.positions;
    return s;
}

bool overlaps(const void* a, size_t an, const void* b, size_t bn) {
    if (!a || !b || !an || !bn) return false;
    const auto x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + bn && y < x + an;
}

// ---- kernel launch helpers --------------------------------------------------------

template <typename T>
size_t smem_vinv(const Plan& p) { return 4 * p.Nj * dev::kVinvModes * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_y(const Plan& p) { return (p.Ny + 2 * dev::kYG * p.Ny) * sizeof(dev::cx<T>); }
inline size_t x_len(const Plan& p) { return p.Nx % 2 == 0 ? p.Nx / 2 : p.Nx; }
template <typename T>
size_t smem_xflux(const Plan& p) {
    const size_t nt = p.targets.count, L = x_len(p);
    return (L + p.Nx + 16 * L) * sizeof(dev::cx<T>) + (3 + nt) * p.Nx * sizeof(T);
}
template <typename T>
size_t smem_xc2r(const Plan& p, int nch) { return (x_len(p) + p.Nx + nch * p.kxColumns + 8 * x_len(p)) * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_xr2c(const Plan& p) { return (x_len(p) + p.Nx + 8 * x_len(p)) * sizeof(dev::cx<T>) + 4 * p.Nx * sizeof(T); }
template <typename T>
size_t smem_vfwd(const Plan& p, int nch) { return nch * p.zHalf * dev::kVfwdModes * sizeof(dev::cx2t<T>); }

// The dynamic shared-memory cap is a process-wide attribute of each kernel,
// not of a handle: only ever raise it, so a handle created for a smaller grid
// cannot shrink the cap below what a live handle for a larger grid launches with.
std::mutex g_smem_mutex;
template <typename K>
cudaError_t raise_smem_limit(K* kernel, int bytes) {
    std::lock_guard<std::mutex> lock(g_smem_mutex);
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, reinterpret_cast<const void*>(kernel));
    if (e != cudaSuccess) return e;
    if (a.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <typename T>
cudaError_t set_smem_limits(const Plan& p) {
    cudaError_t e;
#define WV_SET(kernel, bytes)                                                                                   \
    e = raise_smem_limit(kernel, static_cast<int>(bytes)); \
    if (e != cudaSuccess) return e;
    WV_SET((dev::k_vinv<T, true>), smem_vinv<T>(p));
    WV_SET((dev::k_vinv<T, false>), smem_vinv<T>(p));
    WV_SET((dev::k_yinv<T>), smem_y<T>(p));
    WV_SET((dev::k_yfwd<T>), smem_y<T>(p));
    WV_SET((dev::k_xflux<T>), smem_xflux<T>(p));
    WV_SET((dev::k_xc2r_fields<T>), smem_xc2r<T>(p, 4));
    WV_SET((dev::k_xr2c_fields<T>), smem_xr2c<T>(p));
    WV_SET((dev::k_vfwd<T, true>), smem_vfwd<T>(p, 4));
    WV_SET((dev::k_vfwd<T, false>), smem_vfwd<T>(p, 4));
    if (p.fz.N > 0) {
        WV_SET((dev::k_vinv_fft<T, true>), dev::smem_vinv_fft<T>(static_cast<int>(p.Nj), p.fz.N, dev::VzShape<T, true>::modes));
        WV_SET((dev::k_vinv_fft<T, false>), dev::smem_vinv_fft<T>(static_cast<int>(p.Nj), p.fz.N, dev::VzShape<T, false>::modes));
        WV_SET((dev::k_vfwd_fft<T, true>), dev::smem_vfwd_fft<T>(p.fz.N));
    }
#undef WV_SET
    return cudaSuccess;
}

inline unsigned cdiv(size_t a, size_t b) { return static_cast<unsigned>((a + b - 1) / b); }

// ---- warp-FFT dispatch -------------------------------------------------------------
// y lines of Ny = 32*R and x rows of Nx = 64*R run on register-resident warp
// FFTs; other lengths use the shared-memory Stockham kernels.

template <typename T>
inline int warp_ry(const Plan& p, bool ignoreChoice = false) {
    // FP64 stays on the shared-memory radix-4 Stockham kernels: on the FP64 pipe
    // the radix-2 shuffle stages (64-bit shuffles, the twiddle product evaluated
    // in every lane) cost more than the smem round trips they replace.  Paired
    // FP32 takes the register lines up to 256 points (8 values per lane; 2.7 %
    // faster per flux at 256x256x129, 14 % at 128x128x65) and the Stockham
    // kernel for 512 (16 values per lane: 3 % slower there).
    if (std::is_same<T, double>::value || (p.stockhamY && !ignoreChoice) || p.Ny % 32 != 0) return 0;
    const int r = static_cast<int>(p.Ny / 32);
    const int rmax = sizeof(T) == 8 ? 8 : 16;
    return ((r == 1 || r == 2 || r == 3 || r == 4 || r == 6 || r == 8 || r == 16) && r <= rmax) ? r : 0;
}
template <typename T>
inline int warp_rx(const Plan& p, bool ignoreChoice = false) {
    if (std::is_same<T, double>::value || (p.stockhamX && !ignoreChoice) || p.Nx % 64 != 0) return 0;
    const int r = static_cast<int>(p.Nx / 64);
    const int rmax = sizeof(T) == 8 ? 4 : 8;  // register budget of the fused x row
    return ((r == 1 || r == 2 || r == 3 || r == 4 || r == 6 || r == 8) && r <= rmax) ? r : 0;
}
// The flux's vertical FFT lines (2 (Nz - 1) = 32 R points) on warp registers:
// mixed and FP32X2 handles (FP32X2 up to 256 points), otherwise the Stockham
// kernels of wv_vfft.cuh.
template <typename T>
inline int warp_rz(const Plan& p) {
    if (std::is_same<T, double>::value || p.fz.N == 0 || p.fz.N % 32 != 0) return 0;
    const int r = p.fz.N / 32;
    const int rmax = sizeof(T) == 8 ? 8 : 16;
    return ((r == 1 || r == 2 || r == 3 || r == 4 || r == 6 || r == 8 || r == 16) && r <= rmax) ? r : 0;
}
template <typename T>
size_t smem_y_w(const Plan& p) { return (p.Ny + p.Ny * dev::kWG) * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_xflux_w(const Plan& p) {
    const size_t L = p.Nx / 2;
    const size_t stage = 2 * static_cast<size_t>(dev::xstage_len(static_cast<int>(p.kxColumns)));
    return (3 * L + dev::kWG * (L + stage)) * sizeof(dev::cx<T>);
}
template <typename T>
size_t smem_xc2r_w(const Plan& p, int nch) {
    const size_t L = p.Nx / 2;
    return (3 * L + dev::kWG * (nch * p.kxColumns + L)) * sizeof(dev::cx<T>);
}
template <typename T>
size_t smem_xr2c_w(const Plan& p) { const size_t L = p.Nx / 2; return (3 * L + dev::kWG * L) * sizeof(dev::cx<T>); }

#define WV_RSWITCH_Y(R, BODY)                                             \
    switch (R) {                                                          \
        case 1: { constexpr int RR = 1; BODY; } break;                    \
        case 2: { constexpr int RR = 2; BODY; } break;                    \
        case 3: { constexpr int RR = 3; BODY; } break;                    \
        case 4: { constexpr int RR = 4; BODY; } break;                    \
        case 6: { constexpr int RR = 6; BODY; } break;                    \
        case 8: { constexpr int RR = 8; BODY; } break;                    \
        case 16: { constexpr int RR = 16; BODY; } break;                  \
        default: break;                                                   \
    }
#define WV_RSWITCH_X(T, R, BODY)                                          \
    switch (R) {                                                          \
        case 1: { constexpr int RR = 1; BODY; } break;                    \
        case 2: { constexpr int RR = 2; BODY; } break;                    \
        case 3: { constexpr int RR = 3; BODY; } break;                    \
        case 4: { constexpr int RR = 4; BODY; } break;                    \
        case 6: { if constexpr (sizeof(T) == 4) { constexpr int RR = 6; BODY; } } break; \
        case 8: { if constexpr (sizeof(T) == 4) { constexpr int RR = 8; BODY; } } break; \
        default: break;                                                   \
    }

template <typename T>
cudaError_t set_smem_limits_w(const Plan& p) {
    cudaError_t e = cudaSuccess;
    const int ry = warp_ry<T>(p, true), rx = warp_rx<T>(p, true);
    WV_RSWITCH_Y(ry, {
        e = raise_smem_limit(dev::k_yinv_w<T, RR>, (int)smem_y_w<T>(p));
        if (e == cudaSuccess)
            e = raise_smem_limit(dev::k_yfwd_w<T, RR>, (int)smem_y_w<T>(p));
    });
    if (e != cudaSuccess) return e;
    if constexpr (!std::is_same<T, double>::value) {
        const int rz = warp_rz<T>(p);
        WV_RSWITCH_Y(rz, {
            e = raise_smem_limit(dev::k_vinv_wfft<T, RR>, (int)dev::smem_vinv_wfft<T>(static_cast<int>(p.Nj), p.fz.N));
            if (e == cudaSuccess) e = raise_smem_limit(dev::k_vfwd_wfft<T, RR>, (int)dev::smem_vfwd_wfft<T>(p.fz.N));
        });
        if (e != cudaSuccess) return e;
    }
    WV_RSWITCH_X(T, rx, {
        e = raise_smem_limit(dev::k_xflux_w<T, RR>, (int)smem_xflux_w<T>(p));
        if (e == cudaSuccess)
            e = raise_smem_limit(dev::k_xc2r_fields_w<T, RR>, (int)smem_xc2r_w<T>(p, 4));
        if (e == cudaSuccess)
            e = raise_smem_limit(dev::k_xr2c_fields_w<T, RR>, (int)smem_xr2c_w<T>(p));
    });
    return e;
}

template <typename T>
void launch_yinv(wv_handle* h, const dev::YInvMap& map, const dev::cx<T>* z, dev::cx<T>* y, cudaStream_t s,
                 const dev::DescDev* over = nullptr) {
    const Plan& p = h->plan;
    const dev::DescDev& dd = over ? *over : h->dd;
    const int ry = warp_ry<T>(p);
    if (ry) {
        const dim3 grid(cdiv(p.kxColumns, dev::kWG), dd.zTotal, map.nOut);
        WV_RSWITCH_Y(ry, (dev::k_yinv_w<T, RR><<<grid, 256, smem_y_w<T>(p), s>>>(dd, map, z, y)));
        return;
    }
    dev::k_yinv<T><<<dim3(cdiv(p.kxColumns, dev::kYG), dd.zTotal), 256, smem_y<T>(p), s>>>(dd, map, z, 0, y);
}

template <typename T>
void launch_yfwd(wv_handle* h, const dev::cx<T>* ps, int nch, dev::cx<T>* f, cudaStream_t s) {
    const Plan& p = h->plan;
    const int ry = warp_ry<T>(p);
    if (ry) {
        const dim3 grid(cdiv(p.kxColumns, dev::kWG), h->dd.zTotal, nch);
        WV_RSWITCH_Y(ry, (dev::k_yfwd_w<T, RR><<<grid, 256, smem_y_w<T>(p), s>>>(h->dd, ps, nch, f)));
        return;
    }
    dev::k_yfwd<T><<<dim3(cdiv(p.kxColumns, dev::kYG), h->dd.zTotal, nch), 256, smem_y<T>(p), s>>>(h->dd, ps, nch, f);
}

template <typename T>
void launch_xflux(wv_handle* h, const dev::cx<T>* y, dev::cx<T>* ps, unsigned long long* speed, cudaStream_t s,
                  void* physOut = nullptr, double* advOut = nullptr, const double* advIn = nullptr) {
    const Plan& p = h->plan;
    const int rx = warp_rx<T>(p);
    if (rx) {
        const dim3 grid(cdiv(p.Ny, dev::kWG), h->dd.zTotal);
        WV_RSWITCH_X(T, rx, (dev::k_xflux_w<T, RR><<<grid, 256, smem_xflux_w<T>(p), s>>>(h->dd, y, ps, speed,
                                                                                           static_cast<dev::cx<T>*>(physOut),
                                                                                           advOut, advIn)));
        return;
    }
    dev::k_xflux<T><<<dim3(p.Ny, h->dd.zTotal), 256, smem_xflux<T>(p), s>>>(h->dd, y, ps, speed, static_cast<T*>(physOut),
                                                                           advOut, advIn);
}

template <typename T>
void launch_xc2r(wv_handle* h, const dev::cx<T>* y, double* fields, cudaStream_t s, int nch = 4,
                 const dev::DescDev* over = nullptr) {
    const Plan& p = h->plan;
    const dev::DescDev& dd = over ? *over : h->dd;
    const int rx = warp_rx<T>(p);
    if (rx) {
        const dim3 grid(cdiv(p.Ny, dev::kWG), dd.zTotal);
        WV_RSWITCH_X(T, rx, (dev::k_xc2r_fields_w<T, RR><<<grid, 256, smem_xc2r_w<T>(p, 4), s>>>(dd, y, nch, fields)));
        return;
    }
    dev::k_xc2r_fields<T><<<dim3(p.Ny, dd.zTotal), 256, smem_xc2r<T>(p, 4), s>>>(dd, y, nch, fields);
}

template <typename T>
void launch_xr2c(wv_handle* h, const double* fields, int nch, dev::cx<T>* ps, cudaStream_t s) {
    const Plan& p = h->plan;
    const int rx = warp_rx<T>(p);
    if (rx) {
        const dim3 grid(cdiv(p.Ny, dev::kWG), h->dd.zTotal);
        WV_RSWITCH_X(T, rx, (dev::k_xr2c_fields_w<T, RR><<<grid, 256, smem_xr2c_w<T>(p), s>>>(h->dd, fields, nch, ps)));
        return;
    }
    dev::k_xr2c_fields<T><<<dim3(p.Ny, h->dd.zTotal), 256, smem_xr2c<T>(p), s>>>(h->dd, fields, nch, ps);
}

// The flux's vertical inverse transform with the handle's kernel choice: the
// tensor-core kernels (mixed: split-BF16; FP32X2: digit slices, with the
// y-spectra buffer yScratch as its scratch), the FFTs of the even / odd
// extension or the dense folded contraction.
template <typename T>
void launch_vinv_flux(wv_handle* h, double elapsed, const double* Ap, const double* Am, const double* A0, dev::cx<T>* z,
                      unsigned long long* speed, dev::cx<T>* yScratch, cudaStream_t s) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    auto* y = yScratch;
    if constexpr (sizeof(T) == 4) {
        if (h->vinvKind == WV_VERTICAL_TENSOR_CORES) {
            dev::k_vinv_tc<<<dim3(cdiv(p.Nkl, dev::kTcModes), d.members), dev::kTcThreads, h->tcSmem, s>>>(
                d, Ap, Am, A0, elapsed, reinterpret_cast<float2*>(z), speed);
            return;
        }
    } else if constexpr (std::is_same<T, dev::ff>::value) {
        if (h->vinvKind == WV_VERTICAL_TENSOR_CORES) {
            dev::k_vinv_tcx<<<dim3(cdiv(p.Nkl, dev::kTcModes), d.members), dev::kTcThreads, h->tcxSmem, s>>>(
                d, Ap, Am, A0, elapsed, z, speed, reinterpret_cast<dev::ff*>(y));
            return;
        }
    }
    if (h->vinvKind == WV_VERTICAL_FFT && warp_rz<T>(p)) {
        if constexpr (!std::is_same<T, double>::value) {
            const dim3 grid(cdiv(p.Nkl, dev::kVwWarps / 4), d.members);
            const size_t sm = dev::smem_vinv_wfft<T>(static_cast<int>(p.Nj), p.fz.N);
            WV_RSWITCH_Y(warp_rz<T>(p), (dev::k_vinv_wfft<T, RR><<<grid, 256, sm, s>>>(d, Ap, Am, A0, elapsed, z, speed)));
        }
    } else if (h->vinvKind == WV_VERTICAL_FFT) {
        constexpr int modes = dev::VzShape<T, true>::modes;
        dev::k_vinv_fft<T, true><<<dim3(cdiv(p.Nkl, modes), d.members), 256,
                                    dev::smem_vinv_fft<T>(static_cast<int>(p.Nj), p.fz.N, modes), s>>>(d, Ap, Am, A0, elapsed, z, speed);
    } else {
        dev::k_vinv<T, true><<<dim3(cdiv(p.Nkl, dev::kVinvModes), d.members), 256, smem_vinv<T>(p), s>>>(d, Ap, Am, A0, elapsed, z, speed);
    }
}

// Device scratch of one flux: the z-grid, y-spectra, product and gathered
// spectra buffers and the max-speed counter.  The handle's own buffers by
// default; the static array for wv_nonlinear_flux_device_noalloc.
struct FluxScratch {
    void* z;
    void* y;
    void* p;
    void* f;
    unsigned long long* maxSpeed;
};

// One nonlinear flux (+ adaptive damping when requested) on device buffers.
// physOut, when given, receives the x pass's real rows (U, V, W and the
// derivatives of every target) for the adjoint to reuse.  scratch, when given,
// replaces the handle's scratch buffers (the kernel choice stays the handle's).
template <typename T>
cudaError_t launch_flux(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                        double* Fp, double* Fm, double* F0, bool damping, cudaStream_t s, void* physOut = nullptr,
                        double* advOut = nullptr, const double* advIn = nullptr, const FluxScratch* scratch = nullptr) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    const double elapsed = t - t0;
    if (h->failLaunchAfter >= 0 && h->failLaunchAfter-- == 0) {  // test hook: fail before any launch
        h->injectedFailure = true;
        return cudaErrorLaunchFailure;
    }
    const FluxScratch sc = scratch ? *scratch : FluxScratch{h->zspec, h->yspec, h->pspec, h->fspec, h->maxSpeed};
    auto* z = static_cast<dev::cx<T>*>(sc.z);
    auto* y = static_cast<dev::cx<T>*>(sc.y);
    auto* ps = static_cast<dev::cx<T>*>(sc.p);
    auto* f = static_cast<dev::cx<T>*>(sc.f);
    const int nt = p.targets.count;
    const bool inst = h->instrument;
    // max |u_h| is reduced only when adaptive damping consumes it
    unsigned long long* speed = damping ? sc.maxSpeed : nullptr;
    if (inst) cudaEventRecord(h->ev[0], s);
    launch_vinv_flux<T>(h, elapsed, Ap, Am, A0, z, speed, y, s);
    if (inst) cudaEventRecord(h->ev[1], s);
    dev::YInvMap map{};
    map.nOut = 4 + 2 * nt;
    for (int c = 0; c < 4; ++c) { map.src[c] = c; map.mulL[c] = 0; }
    for (int t2 = 0; t2 < nt; ++t2) {
        map.src[4 + t2] = p.targets.q[t2]; map.mulL[4 + t2] = 1;            // q_y = i l q
        map.src[4 + nt + t2] = 4 + t2;     map.mulL[4 + nt + t2] = 0;        // q_z
    }
    launch_yinv<T>(h, map, z, y, s);
    if (inst) cudaEventRecord(h->ev[2], s);
    launch_xflux<T>(h, y, ps, speed, s, physOut, advOut, advIn);
    if (inst) cudaEventRecord(h->ev[3], s);
    launch_yfwd<T>(h, ps, nt, f, s);
    if (inst) cudaEventRecord(h->ev[4], s);
    bool fwdTC = false;  // forward transform launched by a specialised kernel
    if constexpr (sizeof(T) == 4) {
        if (h->vfwdKind == WV_VERTICAL_TENSOR_CORES) {
            dev::k_vfwd_tc<<<dim3(cdiv(p.Nkl, dev::kTcModes), d.members), dev::kTcThreads, h->tcFwdSmem, s>>>(
                d, reinterpret_cast<const float2*>(f), elapsed, Ap, Am, A0, speed, damping ? 1 : 0, Fp, Fm, F0);
            fwdTC = true;
        }
    }
    if (!fwdTC && h->vfwdKind == WV_VERTICAL_FFT && warp_rz<T>(p)) {
        if constexpr (!std::is_same<T, double>::value) {
            const dim3 grid(cdiv(p.Nkl, dev::kVwWarps / 2), d.members);
            const size_t sm = dev::smem_vfwd_wfft<T>(p.fz.N);
            WV_RSWITCH_Y(warp_rz<T>(p), (dev::k_vfwd_wfft<T, RR><<<grid, 256, sm, s>>>(d, f, nt, elapsed, Ap, Am, A0, speed,
                                                                                          damping ? 1 : 0, Fp, Fm, F0)));
        }
        fwdTC = true;
    }
    if (!fwdTC && h->vfwdKind == WV_VERTICAL_FFT) {
        dev::k_vfwd_fft<T, true><<<dim3(cdiv(p.Nkl, dev::vf_modes<T>()), d.members), 256, dev::smem_vfwd_fft<T>(p.fz.N), s>>>(
            d, f, nt, elapsed, Ap, Am, A0, speed, damping ? 1 : 0, Fp, Fm, F0);
        fwdTC = true;  // forward transform launched
    }
    if (!fwdTC)
        dev::k_vfwd<T, true><<<dim3(cdiv(p.Nkl, dev::kVfwdModes), d.members), 256, smem_vfwd<T>(p, nt), s>>>(
            d, f, nt, elapsed, Ap, Am, A0, speed, damping ? 1 : 0, Fp, Fm, F0);
    h->metrics.kernel_launches += 5;
    cudaError_t e = cudaGetLastError();
    if (inst && e == cudaSuccess) {
        cudaEventRecord(h->ev[5], s);
        e = cudaEventSynchronize(h->ev[5]);
        float ms[5] = {};
        for (int i = 0; i < 5 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&ms[i], h->ev[i], h->ev[i + 1]);
        h->stages.vertical_inverse_ms += ms[0];
        h->stages.y_inverse_ms += ms[1];
        h->stages.x_products_ms += ms[2];
        h->stages.y_forward_ms += ms[3];
        h->stages.vertical_forward_ms += ms[4];
        h->stages.fluxes += 1;
    }
    return e;
}

// ---- F-grid scalar advection ------------------------------------------------------
// Full-spectrum copy of the handle's descriptor (every (kx, ky) row active,
// pos = kx Ny + ky), the scalar pipeline's row wavenumbers (k = 0 at an even-Nx
// Nyquist column, l by signed mode), the per-position flags (bit 0
// self-conjugate row, bit 1 kept by the antialias) and the vertical-derivative
// matrix (kernel.cpp:1066-1110, 466-471).
int ensure_scalar(wv_handle* h) {
    if (h->scalarReady) return WV_SUCCESS;
    const Descriptor& d = h->desc;
    const Plan& p = h->plan;
    const size_t Nx = p.Nx, Ny = p.Ny, Nz = p.Nz, NxHalf = Nx / 2 + 1, P = NxHalf * Ny;
    if (Nz < 3) return fail(h, WV_UNSUPPORTED_OPERATION, "F-grid scalar advection needs Nz >= 3.");
    std::vector<int32_t> posKy(P), colStart(NxHalf + 1), ymap(NxHalf * Ny);
    for (size_t kx = 0; kx <= NxHalf; ++kx) colStart[kx] = static_cast<int32_t>(kx * Ny);
    for (size_t q = 0; q < P; ++q) posKy[q] = static_cast<int32_t>(q % Ny);
    for (size_t q = 0; q < NxHalf * Ny; ++q) ymap[q] = static_cast<int32_t>(q);
    const double pi = 3.141592653589793238462643383279502884;
    std::vector<double> rowK(NxHalf), rowL(Ny);
    for (size_t kx = 0; kx < NxHalf; ++kx)
        rowK[kx] = (Nx % 2 == 0 && kx == Nx / 2) ? 0.0 : 2.0 * pi * static_cast<double>(kx) / d.c.Lx;
    for (size_t ky = 0; ky < Ny; ++ky) {
        const long long lm = ky < (Ny + 1) / 2 ? static_cast<long long>(ky) : static_cast<long long>(ky) - static_cast<long long>(Ny);
        rowL[ky] = 2.0 * pi * static_cast<double>(lm) / d.c.Ly;
    }
    std::vector<unsigned char> flags(P, 0);
    auto posOfRow = [&](uint64_t row) { const size_t kx = row % NxHalf, ky = row / NxHalf; return kx * Ny + ky; };
    for (uint64_t r : d.selfConjugateRows) flags[posOfRow(r)] |= 1;
    for (uint64_t r : d.storageRow) flags[posOfRow(r)] |= 2;
    for (uint64_t r : d.completionRows) flags[posOfRow(r)] |= 2;
    for (uint64_t r : d.completionSources) flags[posOfRow(r)] |= 2;
    // D[z][z'] = sum_{j=1}^{Nz-2} 2 sin(pi j z/(Nz-1)) (-m_j / 2) / (Nz-1) C[j][z'], interior z only;
    // C = the unnormalized DCT-I, m_j = pi j / Lz
    std::vector<double> D(Nz * Nz, 0.0);
    const long long Np = static_cast<long long>(Nz) - 1;
    auto sinpi = [&](long long a) { return std::sin(pi * static_cast<double>(a % (2 * Np)) / static_cast<double>(Np)); };
    auto cospi = [&](long long a) { return std::cos(pi * static_cast<double>(a % (2 * Np)) / static_cast<double>(Np)); };
    for (size_t z = 1; z + 1 < Nz; ++z)
        for (size_t zp = 0; zp < Nz; ++zp) {
            double acc = 0.0;
            for (size_t j = 1; j + 1 < Nz; ++j) {
                const double C = zp == 0 ? 1.0 : (zp == Nz - 1 ? ((j % 2) ? -1.0 : 1.0) : 2.0 * cospi(static_cast<long long>(j * zp)));
                const double mj = pi * static_cast<double>(j) / d.c.Lz;
                acc += 2.0 * sinpi(static_cast<long long>(j * z)) * (-0.5 * mj) * (1.0 / static_cast<double>(Np)) * C;
            }
            D[z * Nz + zp] = acc;
        }
    dev::DescDev sd = h->dd;
    sd.kxColumns = static_cast<int>(NxHalf);
    sd.positions = static_cast<int>(P);
    sd.members = 1;
    sd.zTotal = static_cast<int>(Nz);
    sd.c2rUseK = 0;
    cudaError_t e = cudaSuccess;
    auto up = [&](const auto& v, auto** dst) { if (e == cudaSuccess) e = upload(h, v, dst); };
    up(posKy, &sd.posKy);
    up(colStart, &sd.colStart);
    up(ymap, &sd.ymap);
    const unsigned char* fl = nullptr;
    up(flags, &fl);
    h->scalarFlags = fl;
    const size_t cb = 2 * elem_size(h->precision);
    auto upT = [&](const std::vector<double>& v, const void** dst) {
        if (e != cudaSuccess) return;
        if (h->precision == WV_PRECISION_FP64) { const double* q = nullptr; e = upload(h, v, &q); *dst = q; }
        else if (h->precision == WV_PRECISION_FP32X2) {
            std::vector<float> f(2 * v.size());  // (hi, lo) pairs
            for (size_t i = 0; i < v.size(); ++i) {
                const dev::ff x(v[i]);
                f[2 * i] = x.hi;
                f[2 * i + 1] = x.lo;
            }
            const float* q = nullptr; e = upload(h, f, &q); *dst = q;
        } else { const std::vector<float> f = cast<float>(v); const float* q = nullptr; e = upload(h, f, &q); *dst = q; }
    };
    upT(rowK, &sd.tRowK);
    upT(rowL, &sd.tRowL);
    upT(D, &h->scalarD);
    const size_t R = Nx * Ny * Nz;
    if (e == cudaSuccess) e = alloc(h, 3 * Nz * Ny * NxHalf * cb, &h->scalarP);
    if (e == cudaSuccess) e = alloc(h, 4 * Nz * P * cb, &h->scalarF);
    void* g = nullptr;
    if (e == cudaSuccess) { e = alloc(h, 3 * R * sizeof(double), &g); h->scalarGrad = static_cast<double*>(g); }
    if (e == cudaSuccess) { e = alloc(h, R * sizeof(double), &g); h->scalarRhs = static_cast<double*>(g); }
    // shared memory of the full-width c2r (kx_columns = NxHalf) and of the derivative kernel
    const size_t L = x_len(p);
    const size_t smC2R = (L + Nx + 3 * NxHalf + 8 * L) * cb;
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64    ? raise_smem_limit(dev::k_xc2r_fields<double>, static_cast<int>(smC2R))
            : h->precision == WV_PRECISION_MIXED ? raise_smem_limit(dev::k_xc2r_fields<float>, static_cast<int>(smC2R))
                                                 : raise_smem_limit(dev::k_xc2r_fields<dev::ff>, static_cast<int>(smC2R));
    const size_t smD = Nz * dev::kScalarCols * cb;
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64    ? raise_smem_limit(dev::k_scalar_derivs<double>, static_cast<int>(smD))
            : h->precision == WV_PRECISION_MIXED ? raise_smem_limit(dev::k_scalar_derivs<float>, static_cast<int>(smD))
                                                 : raise_smem_limit(dev::k_scalar_derivs<dev::ff>, static_cast<int>(smD));
    if (e != cudaSuccess) return cuda_fail(h, e, "scalar advection set-up");
    h->sd = sd;
    h->scalarReady = true;
    h->metrics.device_bytes = h->deviceBytes;
    return WV_SUCCESS;
}

// advectFGridScalar (kernel.cpp:1032-1138) on the shared-memory FFT kernels.
template <typename T>
cudaError_t launch_scalar_advection(wv_handle* h, const double* scalar, const double* adv, bool antialias, double* rhs,
                                    cudaStream_t s) {
    const Plan& p = h->plan;
    const dev::DescDev& sd = h->sd;
    const int Ny = static_cast<int>(p.Ny), Nz = static_cast<int>(p.Nz), KX = sd.kxColumns, P = sd.positions;
    const size_t R = p.Nx * p.Ny * p.Nz, L = x_len(p);
    const double hs = 1.0 / static_cast<double>(p.Nx * p.Ny);
    auto* sp = static_cast<dev::cx<T>*>(h->scalarP);
    auto* sf = static_cast<dev::cx<T>*>(h->scalarF);
    const auto* D = static_cast<const T*>(h->scalarD);
    const size_t cb = sizeof(dev::cx<T>);
    const size_t smR2C = (L + p.Nx + 8 * L) * cb + 4 * p.Nx * sizeof(T);
    const size_t smC2R3 = (L + p.Nx + 3 * KX + 8 * L) * cb, smC2R1 = (L + p.Nx + 1 * KX + 8 * L) * cb;
    const unsigned gridE = static_cast<unsigned>(std::min<size_t>((R + 255) / 256, wvgpu::grid_cap(16)));
    // x r2c, y forward FFT of the scalar (channel 3 of sf), column derivatives (channels 0..2)
    dev::k_xr2c_fields<T><<<dim3(Ny, Nz), 256, smR2C, s>>>(sd, scalar, 1, sp);
    dev::cx<T>* sf3 = sf + (size_t)3 * Nz * P;
    dev::k_yfwd<T><<<dim3(cdiv(KX, dev::kYG), Nz, 1), 256, smem_y<T>(p), s>>>(sd, sp, 1, sf3);
    dev::k_scalar_derivs<T><<<cdiv(P, dev::kScalarCols), 256, Nz * dev::kScalarCols * cb, s>>>(sd, sf3, D, h->scalarFlags, hs, sf);
    dev::YInvMap map{};
    map.nOut = 3;
    for (int c = 0; c < 3; ++c) { map.src[c] = c; map.mulL[c] = 0; }
    dev::k_yinv<T><<<dim3(cdiv(KX, dev::kYG), Nz), 256, smem_y<T>(p), s>>>(sd, map, sf, 0, sp);
    dev::k_xc2r_fields<T><<<dim3(Ny, Nz), 256, smC2R3, s>>>(sd, sp, 3, h->scalarGrad);
    dev::k_scalar_rhs<<<gridE, 256, 0, s>>>(h->scalarGrad, adv, R, rhs);
    h->metrics.kernel_launches += 6;
    if (antialias) {
        dev::k_xr2c_fields<T><<<dim3(Ny, Nz), 256, smR2C, s>>>(sd, rhs, 1, sp);
        dev::k_yfwd<T><<<dim3(cdiv(KX, dev::kYG), Nz, 1), 256, smem_y<T>(p), s>>>(sd, sp, 1, sf);
        dev::k_scalar_mask<T><<<static_cast<unsigned>(std::min<size_t>((size_t(Nz) * P + 255) / 256, wvgpu::grid_cap(16))), 256, 0, s>>>(
            sd, sf, h->scalarFlags, hs);
        dev::YInvMap m1{};
        m1.nOut = 1;
        m1.src[0] = 0; m1.mulL[0] = 0;
        dev::k_yinv<T><<<dim3(cdiv(KX, dev::kYG), Nz), 256, smem_y<T>(p), s>>>(sd, m1, sf, 0, sp);
        dev::k_xc2r_fields<T><<<dim3(Ny, Nz), 256, smC2R1, s>>>(sd, sp, 1, rhs);
        h->metrics.kernel_launches += 5;
    }
    return cudaGetLastError();
}

// (d/dx, d/dy, d/dz) of field q (0..3 = u, v, w, eta) at the state
// (transformStateFieldDerivatives, kernel.cpp:719-743): the flux's own stages
// with q as the only target -- vinv gives q and q_z, the y pass q (later times
// i k), i l q and q_z, the x pass c2r of the three with i k on the first.
template <typename T>
cudaError_t launch_field_derivatives(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                                     int q, double* out, cudaStream_t s) {
    const Plan& p = h->plan;
    dev::DescDev d = h->dd;
    d.nt = 1;
    d.tq[0] = q;
    d.c2rUseK = 1;
    auto* z = static_cast<dev::cx<T>*>(h->zspec);
    auto* y = static_cast<dev::cx<T>*>(h->yspec);
    dev::k_vinv<T, true><<<dim3(cdiv(p.Nkl, dev::kVinvModes), d.members), 256, smem_vinv<T>(p), s>>>(d, Ap, Am, A0, t - t0, z,
                                                                                                   nullptr);
    dev::YInvMap map{};
    map.nOut = 3;
    map.src[0] = q; map.mulL[0] = 0;
    map.src[1] = q; map.mulL[1] = 1;
    map.src[2] = 4; map.mulL[2] = 0;
    launch_yinv<T>(h, map, z, y, s, &d);
    launch_xc2r<T>(h, y, out, s, 3, &d);
    h->metrics.kernel_launches += 3;
    return cudaGetLastError();
}

// (value, d/dx, d/dy, d/dz) of the F or G field family of (Apm, A0)
// (transformToSpatialDomainWith{F,G}AllDerivatives, kernel.cpp:819-863).
template <typename T>
cudaError_t launch_family_derivatives(wv_handle* h, bool ffamily, const double* Apm, const double* A0, double* out,
                                      cudaStream_t s) {
    const Plan& p = h->plan;
    dev::DescDev d = h->dd;
    d.c2rUseK = 2;  // channel 1: x derivative
    auto* z = static_cast<dev::cx<T>*>(h->zspec);
    auto* y = static_cast<dev::cx<T>*>(h->yspec);
    const size_t sm = p.Nj * dev::kVinvModes * sizeof(dev::cx<T>);
    if (ffamily)
        dev::k_vinv_family<T, true><<<cdiv(p.Nkl, dev::kVinvModes), 256, sm, s>>>(d, Apm, A0, z);
    else
        dev::k_vinv_family<T, false><<<cdiv(p.Nkl, dev::kVinvModes), 256, sm, s>>>(d, Apm, A0, z);
    dev::YInvMap map{};
    map.nOut = 4;
    map.src[0] = 0; map.mulL[0] = 0;   // value
    map.src[1] = 0; map.mulL[1] = 0;   // i k value (in x)
    map.src[2] = 0; map.mulL[2] = 1;   // i l value
    map.src[3] = 1; map.mulL[3] = 0;   // z derivative
    launch_yinv<T>(h, map, z, y, s, &d);
    launch_xc2r<T>(h, y, out, s, 4, &d);
    h->metrics.kernel_launches += 3;
    return cudaGetLastError();
}

// nch = 4: (u, v, w, eta); nch = 3: (u, v, w) (transformWaveVortexToUVW).
template <typename T>
cudaError_t launch_inverse(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                           double* fields, cudaStream_t s, int nch = 4) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    auto* z = static_cast<dev::cx<T>*>(h->zspec);
    auto* y = static_cast<dev::cx<T>*>(h->yspec);
    dev::k_vinv<T, false><<<dim3(cdiv(p.Nkl, dev::kVinvModes), d.members), 256, smem_vinv<T>(p), s>>>(d, Ap, Am, A0, t - t0, z, nullptr);
    dev::YInvMap map{};
    map.nOut = nch;
    for (int c = 0; c < nch; ++c) { map.src[c] = c; map.mulL[c] = 0; }
    launch_yinv<T>(h, map, z, y, s);
    launch_xc2r<T>(h, y, fields, s, nch);
    h->metrics.kernel_launches += 3;
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_forward(wv_handle* h, const double* fields, double t, double t0, double* Ap, double* Am, double* A0,
                           cudaStream_t s) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    const int nch = h->desc.c.is_hydrostatic ? 3 : 4;
    auto* ps = static_cast<dev::cx<T>*>(h->pspec);
    auto* f = static_cast<dev::cx<T>*>(h->fspec);
    launch_xr2c<T>(h, fields, nch, ps, s);
    launch_yfwd<T>(h, ps, nch, f, s);
    dev::k_vfwd<T, false><<<dim3(cdiv(p.Nkl, dev::kVfwdModes), d.members), 256, smem_vfwd<T>(p, nch), s>>>(
        d, f, nch, t - t0, nullptr, nullptr, nullptr, nullptr, 0, Ap, Am, A0);
    h->metrics.kernel_launches += 3;
    return cudaGetLastError();
}

// ---- adjoint ------------------------------------------------------------------------

template <typename T>
size_t smem_vfwd_adj(const Plan& p) { return p.targets.count * p.Nj * dev::kVfwdModes * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_xadj(const Plan& p) {
    const size_t nt = p.targets.count, L = x_len(p);
    return (L + p.Nx + (nt + 4) * p.kxColumns + 16 * L) * sizeof(dev::cx<T>) + (3 + nt + 3) * p.Nx * sizeof(T);
}
template <typename T>
size_t smem_xadj_w(const Plan& p) {
    const size_t L = p.Nx / 2;
    const size_t stage = 2 * static_cast<size_t>(dev::xadj_stage_len(static_cast<int>(L), static_cast<int>(p.kxColumns)));
    return (3 * L + dev::kWG * (L + 4 * p.kxColumns + stage)) * sizeof(dev::cx<T>);
}
template <typename T>
size_t smem_ypair(const Plan& p) { return (p.Ny + 3 * dev::kYG * p.Ny) * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_ypair_w(const Plan& p) { return (p.Ny + 2 * dev::kWG * p.Ny) * sizeof(dev::cx<T>); }
template <typename T>
size_t smem_xr2c_adj(const Plan& p) { return (x_len(p) + p.Nx + 8 * x_len(p)) * sizeof(dev::cx<T>) + 4 * p.Nx * sizeof(T); }
template <typename T>
size_t smem_vinv_adj(const Plan& p, bool flux) {
    return (flux ? 4 + p.targets.count : 4) * p.zHalf * dev::kVinvAdjModes * sizeof(dev::cx2t<T>);
}

template <typename T>
cudaError_t set_smem_limits_adj(const Plan& p) {
    const size_t limit = 227 * 1024;
    if (smem_xadj<T>(p) > limit || smem_vinv_adj<T>(p, true) > limit || smem_vfwd_adj<T>(p) > limit)
        return cudaErrorInvalidConfiguration;
    cudaError_t e;
#define WV_SET(kernel, bytes)                                                                                   \
    e = raise_smem_limit(kernel, static_cast<int>(bytes)); \
    if (e != cudaSuccess) return e;
    WV_SET((dev::k_vfwd_adj<T>), smem_vfwd_adj<T>(p));
    WV_SET((dev::k_xadj<T>), smem_xadj<T>(p));
    WV_SET((dev::k_yfwd_pair<T>), smem_ypair<T>(p));
    {
        const int ry = warp_ry<T>(p, true);  // both variants: the choice can change after set-up
        WV_RSWITCH_Y(ry, e = raise_smem_limit(dev::k_yfwd_pair_w<T, RR>, (int)smem_ypair_w<T>(p)));
        if (e != cudaSuccess) return e;
    }
    {
        const int rx = warp_rx<T>(p, true);
        WV_RSWITCH_X(T, rx, e = raise_smem_limit(dev::k_xadj_w<T, RR>, (int)smem_xadj_w<T>(p)));
        if (e != cudaSuccess) return e;
    }
    WV_SET((dev::k_xr2c_adj<T>), smem_xr2c_adj<T>(p));
    WV_SET((dev::k_vinv_adj<T, true>), smem_vinv_adj<T>(p, true));
    WV_SET((dev::k_vinv_adj<T, false>), smem_vinv_adj<T>(p, false));
    if (p.fz.N > 0) {
        WV_SET((dev::k_vfwd_adj_fft<T>), dev::smem_vadj_fft<T>(p.fz.N));
        WV_SET((dev::k_vinv_adj_fft<T>), dev::smem_vadj_fft<T>(p.fz.N));
        if constexpr (!std::is_same<T, double>::value) {
            WV_RSWITCH_Y(warp_rz<T>(p), {
                e = raise_smem_limit(dev::k_vfwd_adj_wfft<T, RR>, (int)dev::smem_vfwd_adj_wfft<T>(static_cast<int>(p.Nj), p.fz.N));
                if (e == cudaSuccess) e = raise_smem_limit(dev::k_vinv_adj_wfft<T, RR>, (int)dev::smem_vinv_adj_wfft<T>(p.fz.N));
            });
            if (e != cudaSuccess) return e;
        }
    }
#undef WV_SET
    return cudaSuccess;
}

int ensure_adjoint(wv_handle* h) {
    if (h->adjointReady) return WV_SUCCESS;
    const Plan& p = h->plan;
    const cudaError_t lim = h->precision == WV_PRECISION_FP64    ? set_smem_limits_adj<double>(p)
                            : h->precision == WV_PRECISION_MIXED ? set_smem_limits_adj<float>(p)
                                                                 : set_smem_limits_adj<dev::ff>(p);
    if (lim == cudaErrorInvalidConfiguration)
        return fail(h, WV_UNSUPPORTED_OPERATION, "The adjoint kernels need more shared memory than one CTA has for this grid.");
    if (lim != cudaSuccess) return cuda_fail(h, lim, "adjoint set-up");
    const size_t nt = p.targets.count, nIn = 4 + 2 * nt;
    const size_t cb = 2 * elem_size(h->precision);
    cudaError_t e = alloc(h, nt * p.Nz * p.positions * cb, &h->zadj);
    if (e == cudaSuccess) e = alloc(h, p.Nz * nt * p.Ny * p.kxColumns * cb, &h->yadj);
    if (e == cudaSuccess) e = alloc(h, p.Nz * nIn * p.Ny * p.kxColumns * cb, &h->yout);
    if (e == cudaSuccess) e = alloc(h, nIn * p.Nz * p.positions * cb, &h->fadj);
    const size_t stateBytes = 6 * p.M * sizeof(double);
    void* tmp = nullptr;
    for (int i = 1; i < 4 && e == cudaSuccess; ++i) { e = alloc(h, stateBytes, &tmp); h->st[i] = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->kb = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->sb = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->ybacc = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->ybin = static_cast<double*>(tmp); }
    if (e != cudaSuccess) return cuda_fail(h, e, "adjoint workspace");
    h->metrics.device_bytes = h->deviceBytes;
    h->adjointReady = true;
    return WV_SUCCESS;
}

// VJP of the nonlinear flux (no damping) at state A: (Fpb, Fmb, F0b) -> (Apb, Amb, A0b).
// y spectra of the 4+2nt flux input channels at state A (the first two
// stages of the flux) into y.
template <typename T>
void launch_flux_fields(wv_handle* h, double elapsed, const double* Ap, const double* Am, const double* A0, dev::cx<T>* y,
                        cudaStream_t s) {
    const Plan& p = h->plan;
    const int nt = p.targets.count;
    auto* z = static_cast<dev::cx<T>*>(h->zspec);
    launch_vinv_flux<T>(h, elapsed, Ap, Am, A0, z, nullptr, y, s);
    dev::YInvMap map{};
    map.nOut = 4 + 2 * nt;
    for (int c = 0; c < 4; ++c) { map.src[c] = c; map.mulL[c] = 0; }
    for (int t2 = 0; t2 < nt; ++t2) {
        map.src[4 + t2] = p.targets.q[t2]; map.mulL[4 + t2] = 1;
        map.src[4 + nt + t2] = 4 + t2;     map.mulL[4 + nt + t2] = 0;
    }
    launch_yinv<T>(h, map, z, y, s);
    h->metrics.kernel_launches += 2;
}

// physIn, when given, holds the forward x pass's real rows at this state
// (kept by the forward flux); otherwise the forward fields are recomputed.
template <typename T>
cudaError_t launch_flux_vjp(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                            const double* Fpb, const double* Fmb, const double* F0b, double* Apb, double* Amb, double* A0b,
                            cudaStream_t s, const void* physIn = nullptr) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    const double elapsed = t - t0;
    const int nt = p.targets.count, nIn = 4 + 2 * nt;
    auto* za = static_cast<dev::cx<T>*>(h->zadj);
    auto* ya = static_cast<dev::cx<T>*>(h->yadj);
    auto* yo = static_cast<dev::cx<T>*>(h->yout);
    auto* fa = static_cast<dev::cx<T>*>(h->fadj);
    // forward fields of this state
    const dev::cx<T>* y = static_cast<const dev::cx<T>*>(h->yspec);
    if (!physIn) launch_flux_fields<T>(h, elapsed, Ap, Am, A0, static_cast<dev::cx<T>*>(h->yspec), s);
    // adjoint of projection and forward vertical transform, then inverse y FFTs
    bool done = false;  // the vertical forward map launched on warp lines
    if constexpr (!std::is_same<T, double>::value) {
        if (h->vfwdKind == WV_VERTICAL_FFT && warp_rz<T>(p)) {
            const dim3 grid(cdiv(p.Nkl, dev::kVwWarps / 2), d.members);
            const size_t sm = dev::smem_vfwd_adj_wfft<T>(static_cast<int>(p.Nj), p.fz.N);
            WV_RSWITCH_Y(warp_rz<T>(p), (dev::k_vfwd_adj_wfft<T, RR><<<grid, 256, sm, s>>>(d, Fpb, Fmb, F0b, elapsed, za)));
            done = true;
        }
    }
    if (done) {
    } else if (h->vfwdKind == WV_VERTICAL_FFT)
        dev::k_vfwd_adj_fft<T><<<dim3(cdiv(p.Nkl, dev::vf_modes<T>()), d.members), 256, dev::smem_vadj_fft<T>(p.fz.N), s>>>(
            d, Fpb, Fmb, F0b, elapsed, za);
    else
        dev::k_vfwd_adj<T><<<dim3(cdiv(p.Nkl, dev::kVfwdModes), d.members), 256, smem_vfwd_adj<T>(p), s>>>(d, Fpb, Fmb, F0b, elapsed, za);
    dev::YInvMap amap{};
    amap.nOut = nt;
    for (int c = 0; c < nt; ++c) { amap.src[c] = c; amap.mulL[c] = 0; }
    launch_yinv<T>(h, amap, za, ya, s);
    const int rx = warp_rx<T>(p);
    if (rx) {
        const dim3 grid(cdiv(p.Ny, dev::kWG), p.Nz);
        WV_RSWITCH_X(T, rx, (dev::k_xadj_w<T, RR><<<grid, 256, smem_xadj_w<T>(p), s>>>(
                                 d, y, ya, yo, static_cast<const dev::cx<T>*>(physIn))));
    } else {
        dev::k_xadj<T><<<dim3(p.Ny, p.Nz), 256, smem_xadj<T>(p), s>>>(d, y, ya, yo, static_cast<const T*>(physIn));
    }
    // y forward with each target's y-derivative channel folded onto its value channel
    dev::YFwdPairMap pm{};
    pm.nOut = 4 + nt;
    for (int c = 0; c < 4; ++c) { pm.srcA[c] = c; pm.srcB[c] = -1; }
    for (int t2 = 0; t2 < nt; ++t2) {
        pm.srcB[p.targets.q[t2]] = 4 + t2;
        pm.srcA[4 + t2] = 4 + nt + t2;
        pm.srcB[4 + t2] = -1;
    }
    {
        const int ry = warp_ry<T>(p);
        if (ry) {
            const dim3 grid(cdiv(p.kxColumns, dev::kWG), d.zTotal, pm.nOut);
            WV_RSWITCH_Y(ry, (dev::k_yfwd_pair_w<T, RR><<<grid, 256, smem_ypair_w<T>(p), s>>>(d, pm, yo, nIn, fa)));
        } else {
            dev::k_yfwd_pair<T><<<dim3(cdiv(p.kxColumns, dev::kYG), d.zTotal, pm.nOut), 256, smem_ypair<T>(p), s>>>(d, pm, yo,
                                                                                                              nIn, fa);
        }
    }
    bool vdone = false;  // the vertical inverse map launched on warp lines
    if constexpr (!std::is_same<T, double>::value) {
        if (h->vinvKind == WV_VERTICAL_FFT && warp_rz<T>(p)) {
            const dim3 grid(cdiv(p.Nkl, dev::kVwWarps / 4), d.members);
            const size_t sm = dev::smem_vinv_adj_wfft<T>(p.fz.N);
            WV_RSWITCH_Y(warp_rz<T>(p), (dev::k_vinv_adj_wfft<T, RR><<<grid, 256, sm, s>>>(d, fa, elapsed, Apb, Amb, A0b)));
            vdone = true;
        }
    }
    if (vdone) {
    } else if (h->vinvKind == WV_VERTICAL_FFT)
        dev::k_vinv_adj_fft<T><<<dim3(cdiv(p.Nkl, dev::VzLines<T>::value / 4), d.members), 256, dev::smem_vadj_fft<T>(p.fz.N), s>>>(
            d, fa, elapsed, Apb, Amb, A0b);
    else
        dev::k_vinv_adj<T, true><<<dim3(cdiv(p.Nkl, dev::kVinvAdjModes), d.members), 256, smem_vinv_adj<T>(p, true), s>>>(d, fa, nIn, elapsed, Apb, Amb, A0b);
    h->metrics.kernel_launches += 5;
    return cudaGetLastError();
}

// VJP of the inverse transform: fields_bar [4][Nz][Ny][Nx] -> (Apb, Amb, A0b).
template <typename T>
cudaError_t launch_inverse_vjp(wv_handle* h, double t, double t0, const double* fb, double* Apb, double* Amb, double* A0b,
                               cudaStream_t s) {
    const Plan& p = h->plan;
    const auto& d = h->dd;
    auto* ps = static_cast<dev::cx<T>*>(h->pspec);
    auto* fa = static_cast<dev::cx<T>*>(h->fadj);
    dev::k_xr2c_adj<T><<<dim3(p.Ny, p.Nz), 256, smem_xr2c_adj<T>(p), s>>>(d, fb, 4, ps);
    launch_yfwd<T>(h, ps, 4, fa, s);
    dev::k_vinv_adj<T, false><<<dim3(cdiv(p.Nkl, dev::kVinvAdjModes), d.members), 256, smem_vinv_adj<T>(p, false), s>>>(d, fa, 4, t - t0, Apb, Amb, A0b);
    h->metrics.kernel_launches += 3;
    return cudaGetLastError();
}

cudaError_t flux_vjp_any(wv_handle* h, double t, double t0, const double* y, const double* yb, double* out, cudaStream_t s,
                         const void* physIn = nullptr) {
    const size_t M2 = 2 * h->plan.M;
    return h->precision == WV_PRECISION_FP64
               ? launch_flux_vjp<double>(h, t, t0, y, y + M2, y + 2 * M2, yb, yb + M2, yb + 2 * M2, out, out + M2, out + 2 * M2, s, physIn)
               : h->precision == WV_PRECISION_MIXED ? launch_flux_vjp<float>(h, t, t0, y, y + M2, y + 2 * M2, yb, yb + M2, yb + 2 * M2, out, out + M2, out + 2 * M2, s, physIn)
                                                          : launch_flux_vjp<dev::ff>(h, t, t0, y, y + M2, y + 2 * M2, yb, yb + M2, yb + 2 * M2, out, out + M2, out + 2 * M2, s, physIn);
}

cudaError_t flux_any(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* Fp,
                     double* Fm, double* F0, bool damping, cudaStream_t s, void* physOut = nullptr, double* advOut = nullptr,
                     const double* advIn = nullptr) {
    return h->precision == WV_PRECISION_FP64
               ? launch_flux<double>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, damping, s, physOut, advOut, advIn)
               : h->precision == WV_PRECISION_MIXED ? launch_flux<float>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, damping, s, physOut, advOut, advIn)
                                                          : launch_flux<dev::ff>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, damping, s, physOut, advOut, advIn);
}

// Scheduled RHS on contiguous [3][M] complex state/flux buffers.
cudaError_t rhs_contiguous(wv_handle* h, double t, double t0, const double* y, double* k, cudaStream_t s) {
    const size_t M2 = 2 * h->plan.M;
    const bool damping = (h->forcing & WV_FORCING_ADAPTIVE_DAMPING) != 0;
    if (!(h->forcing & WV_FORCING_NONLINEAR_ADVECTION)) {
        // damping only is not a configuration the reference's default schedules produce
        return cudaErrorNotSupported;
    }
    return flux_any(h, t, t0, y, y + M2, y + 2 * M2, k, k + M2, k + 2 * M2, damping, s);
}

// WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462) on the
// contiguous device state h->state.
cudaError_t rk4_step(wv_handle* h, double t, double t0, double dt, cudaStream_t s) {
    const size_t n = 6 * h->plan.M * h->dd.members;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, wvgpu::grid_cap(16)));
    const bool dense = h->rk4Dense && h->denseBuf;
    const size_t nb = n * sizeof(double);
    cudaError_t e;
    if (dense) { e = cudaMemcpyAsync(h->denseBuf, h->state, nb, cudaMemcpyDeviceToDevice, s); if (e != cudaSuccess) return e; }
    e = rhs_contiguous(h, t, t0, h->state, h->kbuf, s); if (e != cudaSuccess) return e;
    if (dense) { e = cudaMemcpyAsync(h->denseBuf + 2 * n, h->kbuf, nb, cudaMemcpyDeviceToDevice, s); if (e != cudaSuccess) return e; }
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 1.0, h->state, 0.5 * dt, h->stage, 1, n);
    e = rhs_contiguous(h, t + 0.5 * dt, t0, h->stage, h->kbuf, s); if (e != cudaSuccess) return e;
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 2.0, h->state, 0.5 * dt, h->stage, 0, n);
    e = rhs_contiguous(h, t + 0.5 * dt, t0, h->stage, h->kbuf, s); if (e != cudaSuccess) return e;
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 2.0, h->state, dt, h->stage, 0, n);
    e = rhs_contiguous(h, t + dt, t0, h->stage, h->kbuf, s); if (e != cudaSuccess) return e;
    if (dense) { e = cudaMemcpyAsync(h->denseBuf + 3 * n, h->kbuf, nb, cudaMemcpyDeviceToDevice, s); if (e != cudaSuccess) return e; }
    dev::k_rk4_finish<<<grid, 256, 0, s>>>(h->acc, h->kbuf, h->state, dt / 6.0, h->state, n);
    if (dense) { e = cudaMemcpyAsync(h->denseBuf + n, h->state, nb, cudaMemcpyDeviceToDevice, s); if (e != cudaSuccess) return e; }
    h->metrics.kernel_launches += 4;
    h->metrics.rk4_steps += 1;
    h->metrics.rhs_evaluations += 4;
    return cudaGetLastError();
}

// Stage states of one WVFixedStepRK4 step from y (contiguous [3][M] complex):
// st1 = y + h/2 k1, st2 = y + h/2 k2, st3 = y + h k3; when yNext is given it
// also receives the step's result with the same arithmetic as rk4_step.
// With ys (four buffers), the x pass's real rows at y, st1, st2 and st3 are
// kept for the step's adjoint (st3's flux then runs even without yNext).
cudaError_t rk4_stages(wv_handle* h, const double* y, double t, double t0, double dt, double* st1, double* st2, double* st3,
                       double* yNext, cudaStream_t s, void* const* ys = nullptr) {
    const size_t n = 6 * h->plan.M;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, wvgpu::grid_cap(16)));
    const size_t M2 = 2 * h->plan.M;
    auto flux = [&](const double* x, double tt, int k) {
        return flux_any(h, tt, t0, x, x + M2, x + 2 * M2, h->kbuf, h->kbuf + M2, h->kbuf + 2 * M2, false, s,
                        ys ? ys[k] : nullptr);
    };
    cudaError_t e = flux(y, t, 0); if (e != cudaSuccess) return e;
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 1.0, y, 0.5 * dt, st1, 1, n);
    e = flux(st1, t + 0.5 * dt, 1); if (e != cudaSuccess) return e;
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 2.0, y, 0.5 * dt, st2, 0, n);
    e = flux(st2, t + 0.5 * dt, 2); if (e != cudaSuccess) return e;
    dev::k_accumulate_and_stage<<<grid, 256, 0, s>>>(h->acc, h->kbuf, 2.0, y, dt, st3, 0, n);
    h->metrics.kernel_launches += 3;
    if (!yNext && ys) { e = flux(st3, t + dt, 3); if (e != cudaSuccess) return e; }
    if (yNext) {
        e = flux(st3, t + dt, 3); if (e != cudaSuccess) return e;
        dev::k_rk4_finish<<<grid, 256, 0, s>>>(h->acc, h->kbuf, y, dt / 6.0, yNext, n);
        h->metrics.kernel_launches += 1;
    }
    return cudaGetLastError();
}

// Backward sweep of one RK4 step given its stage states: yb is the cotangent of
// the state after the step; h->ybacc receives the cotangent before it.
cudaError_t rk4_backward(wv_handle* h, const double* y, const double* st1, const double* st2, const double* st3, double t,
                         double t0, double dt, const double* yb, cudaStream_t s, void* const* ys = nullptr,
                         double* ybOut = nullptr) {
    if (!ybOut) ybOut = h->ybacc;
    const size_t n = 6 * h->plan.M;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((n + 255) / 256, wvgpu::grid_cap(16)));
    cudaError_t e;
    dev::k_lincomb<<<grid, 256, 0, s>>>(h->kb, dt / 6.0, yb, 0.0, nullptr, n);
    e = flux_vjp_any(h, t + dt, t0, st3, h->kb, h->sb, s, ys ? ys[3] : nullptr); if (e != cudaSuccess) return e;
    dev::k_adj_stage<<<grid, 256, 0, s>>>(ybOut, true, h->kb, dt / 3.0, yb, dt, h->sb, n);
    e = flux_vjp_any(h, t + 0.5 * dt, t0, st2, h->kb, h->sb, s, ys ? ys[2] : nullptr); if (e != cudaSuccess) return e;
    dev::k_adj_stage<<<grid, 256, 0, s>>>(ybOut, false, h->kb, dt / 3.0, yb, 0.5 * dt, h->sb, n);
    e = flux_vjp_any(h, t + 0.5 * dt, t0, st1, h->kb, h->sb, s, ys ? ys[1] : nullptr); if (e != cudaSuccess) return e;
    dev::k_adj_stage<<<grid, 256, 0, s>>>(ybOut, false, h->kb, dt / 6.0, yb, 0.5 * dt, h->sb, n);
    e = flux_vjp_any(h, t, t0, y, h->kb, h->sb, s, ys ? ys[0] : nullptr); if (e != cudaSuccess) return e;
    dev::k_accumulate<<<grid, 256, 0, s>>>(ybOut, h->sb, n);
    h->metrics.kernel_launches += 5;
    return cudaGetLastError();
}

// Adjoint of one WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462)
// at state y, stage states recomputed.
cudaError_t rk4_step_vjp(wv_handle* h, const double* y, double t, double t0, double dt, const double* yb, cudaStream_t s) {
    cudaError_t e = rk4_stages(h, y, t, t0, dt, h->st[1], h->st[2], h->st[3], nullptr, s);
    if (e != cudaSuccess) return e;
    return rk4_backward(h, y, h->st[1], h->st[2], h->st[3], t, t0, dt, yb, s);
}

int check_times(wv_handle* h, double t, double t0) {
    if (!std::isfinite(t) || !std::isfinite(t0)) return fail(h, WV_INVALID_CONFIGURATION, "State times must be finite.");
    return WV_SUCCESS;
}

int check_state_flux(wv_handle* h, const double* Ap, const double* Am, const double* A0, double* Fp, double* Fm, double* F0) {
    const char* names[] = {"Ap", "Am", "A0", "Fp", "Fm", "F0"};
    const void* ptrs[] = {Ap, Am, A0, Fp, Fm, F0};
    for (int i = 0; i < 6; ++i)
        if (!ptrs[i]) return fail(h, WV_INVALID_POINTER, std::string(names[i]) + " has a null data pointer.");
    const size_t bytes = h->plan.M * 16;
    const void* outs[] = {Fp, Fm, F0};
    const void* ins[] = {Ap, Am, A0};
    for (int i = 0; i < 3; ++i) {
        for (int j = i + 1; j < 3; ++j)
            if (overlaps(outs[i], bytes, outs[j], bytes)) return fail(h, WV_OVERLAPPING_ARRAYS, "Flux outputs must not overlap.");
        for (const void* in : ins)
            if (overlaps(outs[i], bytes, in, bytes)) return fail(h, WV_OVERLAPPING_ARRAYS, "Flux outputs must not overlap state inputs.");
    }
    return WV_SUCCESS;
}

int finish(wv_handle* h, cudaError_t e, const char* where) {
    if (e != cudaSuccess) return cuda_fail(h, e, where);
    return WV_SUCCESS;
}


// ---- static scratch for callers that cannot allocate ------------------------------
//
// One file-scope device array holds the flux pipeline's scratch for
// wv_nonlinear_flux_device_noalloc.  Every GPU that loads this library keeps
// WV_STATIC_SCRATCH_BYTES resident until the process exits.  In host code the
// array's name is only a host-side stand-in; its device address is looked up
// once per device with cudaGetSymbolAddress, with that device current.

constexpr size_t kStaticScratchBytes = WV_STATIC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_scratch_mutex;
void* g_static_scratch_address[kMaxDevices] = {};

// Device address of g_static_scratch on `device` (the current device).
cudaError_t static_scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_scratch_mutex);
    if (!g_static_scratch_address[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_static_scratch_address[device] = p;
    }
    *out = g_static_scratch_address[device];
    return cudaSuccess;
}

inline size_t round256(size_t n) { return (n + 255) / 256 * 256; }

// Byte offsets of the four scratch buffers and the speed counter inside the
// static array; returns the total size.
size_t static_scratch_layout(const Plan& p, size_t complexBytes, size_t offs[5]) {
    const auto ss = scratch_sizes(p);
    const size_t sizes[5] = {ss.z * complexBytes, ss.y * complexBytes, ss.p * complexBytes, ss.f * complexBytes,
                             sizeof(unsigned long long)};
    size_t off = 0;
    for (int i = 0; i < 5; ++i) { offs[i] = off; off += round256(sizes[i]); }
    return off;
}

}  // namespace

namespace wvgpu {
size_t grid_cap(size_t perSm) {
    static std::atomic<int> sms[64] = {};
    int device = 0;
    cudaGetDevice(&device);
    if (device < 0 || device >= 64) device = 0;
    int n = sms[device].load();
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0) n = 1;
        sms[device].store(n);
    }
    return perSm * static_cast<size_t>(n);
}

const Descriptor& handle_descriptor(const wv_handle* h) { return h->desc; }
int handle_device(const wv_handle* h) { return h->device; }
void* handle_stream(const wv_handle* h) { return h->stream; }
bool handle_is_single_state(const wv_handle* h) { return h->dd.members == 1; }

int scheduled_rhs_with_fields(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                              double* Fp, double* Fm, double* F0, double* fields, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    if (!fields) return fail(h, WV_INVALID_POINTER, "Advection fields pointer must be nonnull.");
    if (!(h->forcing & WV_FORCING_NONLINEAR_ADVECTION))
        return fail(h, WV_UNSUPPORTED_OPERATION, "Integrated observers need the nonlinear advection schedule.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const bool damping = (h->forcing & WV_FORCING_ADAPTIVE_DAMPING) != 0;
    const cudaError_t e = flux_any(h, t, t0, Ap, Am, A0, Fp, Fm, F0, damping, static_cast<cudaStream_t>(stream), nullptr, fields);
    h->metrics.rhs_evaluations++;
    return finish(h, e, "right-hand side");
}
}  // namespace wvgpu

extern "C" {

int wv_describe(const wv_config* config, wv_sizes* sizes, char* message, size_t cap) {
    auto msg = [&](const std::string& m) {
        if (message && cap) { std::strncpy(message, m.c_str(), cap - 1); message[cap - 1] = 0; }
    };
    if (!config) { msg("Configuration pointer is null."); return WV_INVALID_POINTER; }
    Descriptor d;
    Status st = wvgpu::build_descriptor(*config, d);
    if (!st) { msg(st.message); return st.code; }
    Plan p;
    st = wvgpu::build_plan(d, p);
    if (!st) { msg(st.message); return st.code; }
    if (sizes) {
        sizes->Nx = p.Nx; sizes->Ny = p.Ny; sizes->Nz = p.Nz; sizes->Nj = p.Nj; sizes->Nkl = p.Nkl; sizes->NxHalf = p.NxHalf;
        sizes->M = p.M; sizes->active_rows = p.positions; sizes->kx_columns = p.kxColumns;
        const auto s = scratch_sizes(p);
        const size_t R = p.Nx * p.Ny * p.Nz;
        sizes->device_bytes = (s.z + s.y + s.p + s.f) * 16 + 5 * 6 * p.M * sizeof(double) + 4 * R * sizeof(double) +
                              20 * p.M * sizeof(double);
    }
    msg("");
    return WV_SUCCESS;
}

int wv_describe_modes(const wv_config* config, int64_t* kMode, int64_t* lMode, double* omega, uint64_t* rows, uint8_t* conj) {
    if (!config) return WV_INVALID_POINTER;
    Descriptor d;
    Status st = wvgpu::build_descriptor(*config, d);
    if (!st) return st.code;
    if (kMode) std::memcpy(kMode, d.kMode.data(), d.Nkl * sizeof(int64_t));
    if (lMode) std::memcpy(lMode, d.lMode.data(), d.Nkl * sizeof(int64_t));
    if (omega) std::memcpy(omega, d.omega.data(), d.M * sizeof(double));
    if (rows) std::memcpy(rows, d.storageRow.data(), d.Nkl * sizeof(uint64_t));
    if (conj) std::memcpy(conj, d.conjugated.data(), d.Nkl);
    return WV_SUCCESS;
}

void wv_destroy(wv_handle* h) {
    if (!h) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(h->device);
    if (h->stream) { cudaStreamSynchronize(h->stream); cudaStreamDestroy(h->stream); }
    if (h->adjStream) { cudaStreamSynchronize(h->adjStream); cudaStreamDestroy(h->adjStream); }
    for (auto& ev : h->ev) if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : {h->slotReady[0], h->slotReady[1], h->slotFree[0], h->slotFree[1], h->fwdDone})
        if (ev) cudaEventDestroy(ev);
    for (void* p : h->allocations) cudaFree(p);
    g_liveDeviceBytes -= static_cast<long long>(h->deviceBytes);
    cudaSetDevice(prev);
    delete h;
}

// A handle for `members` states of one grid stepped side by side (members = 1
// for the reference's single-state kernel).
static int create_handle(const wv_config* config, int precision, int members, wv_handle** out) {
    if (!out) return WV_INVALID_POINTER;
    *out = nullptr;
    if (!config) return WV_INVALID_POINTER;
    if (precision != WV_PRECISION_FP64 && precision != WV_PRECISION_MIXED && precision != WV_PRECISION_FP32X2)
        return WV_INVALID_CONFIGURATION;
    if (members < 1) return WV_INVALID_CONFIGURATION;
    wv_handle* h = new (std::nothrow) wv_handle();
    if (!h) return WV_ALLOCATION_FAILURE;
    h->precision = precision;
    Status st = wvgpu::build_descriptor(*config, h->desc);
    if (st) st = wvgpu::build_plan(h->desc, h->plan);
    if (!st) { const int code = st.code; delete h; return code; }
    const Descriptor& d = h->desc;
    const Plan& p = h->plan;
    // plane index m*Nz+z rides in gridDim.y (at most 65535)
    if (static_cast<size_t>(members) * p.Nz > 65535) { delete h; return WV_INVALID_CONFIGURATION; }
    cudaGetDevice(&h->device);
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    std::vector<double> damping;
    if (e == cudaSuccess) {
        Status ds = wvgpu::adaptive_damping_operator(d, damping);
        h->hasDamping = static_cast<bool>(ds);
        if (!ds) damping.assign(d.M, 0.0);
    }
    auto& dd = h->dd;
    dd.Nx = p.Nx; dd.Ny = p.Ny; dd.Nz = p.Nz; dd.Nj = p.Nj; dd.Nkl = p.Nkl; dd.NxHalf = p.NxHalf; dd.M = p.M;
    dd.members = members; dd.zTotal = static_cast<int>(members * p.Nz);
    dd.memberStride = static_cast<long long>(6 * p.M);
    dd.positions = p.positions; dd.kxColumns = p.kxColumns; dd.zHalf = p.zHalf;
    dd.nt = p.targets.count;
    for (int i = 0; i < 4; ++i) dd.tq[i] = p.targets.q[i];
    dd.hydrostatic = d.c.is_hydrostatic ? 1 : 0;
    dd.xEven = p.Nx % 2 == 0 ? 1 : 0;
    dd.xLen = static_cast<int>(x_len(p));
    dd.fx.N = p.fx.N; dd.fx.nstages = p.fx.nstages; dd.fy.N = p.fy.N; dd.fy.nstages = p.fy.nstages;
    for (int i = 0; i < dev::kMaxStages; ++i) { dd.fx.radix[i] = p.fx.radix[i]; dd.fy.radix[i] = p.fy.radix[i]; }
    dd.fz.N = p.fz.N; dd.fz.nstages = p.fz.nstages;
    for (int i = 0; i < dev::kMaxStages; ++i) dd.fz.radix[i] = p.fz.radix[i];
    std::vector<int32_t> ymap(p.ymap);
    std::vector<int32_t> posKy(p.posKy), colStart(p.colStart), modeWV(p.modeWV), modePos(p.modePos), modeComp(p.modeCompPos);
    std::vector<double> inertial(d.inertialScale), apmw(d.apmWProjectionPrefactor);
#define WV_UP(vec, field)                                            \
    if (e == cudaSuccess) {                                          \
        e = upload(h, vec, &dd.field);                               \
    }
    WV_UP(d.omega, omega);
    std::vector<double> UAp = interleave(d.UAp), VAp = interleave(d.VAp), WAp = interleave(d.WAp), UA0 = interleave(d.UA0),
                        VA0 = interleave(d.VA0), ApmD = interleave(d.ApmD);
    WV_UP(UAp, UAp); WV_UP(VAp, VAp); WV_UP(WAp, WAp); WV_UP(d.NAp, NAp); WV_UP(UA0, UA0); WV_UP(VA0, VA0); WV_UP(d.NA0, NA0);
    WV_UP(d.A0FromVorticity, A0FromVorticity); WV_UP(d.A0FromBuoyancy, A0FromBuoyancy); WV_UP(d.ApmN, ApmN);
    WV_UP(d.ApmDScaled, ApmDScaled); WV_UP(ApmD, ApmD); WV_UP(damping, damping);
    WV_UP(d.k, k); WV_UP(d.l, l); WV_UP(d.Kh, Kh); WV_UP(d.cosAlpha, cosAlpha); WV_UP(d.sinAlpha, sinAlpha);
    WV_UP(inertial, inertialScale); WV_UP(apmw, apmWPrefactor);
    WV_UP(d.fWaveScale, fWaveScale); WV_UP(d.gWaveScale, gWaveScale); WV_UP(d.Fg, Fg); WV_UP(d.Gg, Gg);
    WV_UP(posKy, posKy); WV_UP(colStart, colStart); WV_UP(ymap, ymap); WV_UP(modeWV, modeWV); WV_UP(modePos, modePos); WV_UP(modeComp, modeCompPos);
    WV_UP(p.modeFlags, modeFlags);
    WV_UP(p.rowK, rowK); WV_UP(p.rowL, rowL);
#undef WV_UP
    // FP32 copies (MIXED) or (hi, lo) pairs (FP32X2) of the arrays the vertical
    // kernels' reduced-precision branches read
    auto to_pairs = [](const std::vector<double>& v) {
        std::vector<float> f(2 * v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            const dev::ff x(v[i]);
            f[2 * i] = x.hi;
            f[2 * i + 1] = x.lo;
        }
        return f;
    };
    if (precision == WV_PRECISION_MIXED || precision == WV_PRECISION_FP32X2) {
        auto upf = [&](const std::vector<double>& v, const float** dst) {
            if (e != cudaSuccess) return;
            const std::vector<float> f = precision == WV_PRECISION_MIXED ? cast<float>(v) : to_pairs(v);
            e = upload(h, f, dst);
        };
        upf(UAp, &dd.fUAp); upf(VAp, &dd.fVAp); upf(WAp, &dd.fWAp); upf(d.NAp, &dd.fNAp);
        upf(UA0, &dd.fUA0); upf(VA0, &dd.fVA0); upf(d.NA0, &dd.fNA0);
    }
    auto upT = [&](const std::vector<double>& v, const void** dst) {
        if (e != cudaSuccess) return;
        if (precision == WV_PRECISION_FP64) {
            const double* q = nullptr; e = upload(h, v, &q); *dst = q;
        } else if (precision == WV_PRECISION_FP32X2) {
            const std::vector<float> f = to_pairs(v);
            const float* q = nullptr; e = upload(h, f, &q); *dst = q;
        } else {
            const std::vector<float> f = cast<float>(v);
            const float* q = nullptr; e = upload(h, f, &q); *dst = q;
        }
    };
    upT(p.Ccos, &dd.Ccos); upT(p.Csin, &dd.Csin); upT(p.CcosM, &dd.CcosM); upT(p.CsinM, &dd.CsinM);
    upT(p.Fcos, &dd.Fcos); upT(p.Fsin, &dd.Fsin); upT(p.twx, &dd.twx); upT(p.twxN, &dd.twxN); upT(p.twy, &dd.twy);
    if (p.fz.N > 0) { upT(p.twz, &dd.twz); upT(std::vector<double>(d.m.begin(), d.m.begin() + p.Nj), &dd.tMz); }
    upT(p.rowK, &dd.tRowK); upT(p.rowL, &dd.tRowL);
    {
        auto transpose = [](const std::vector<double>& a, size_t rows, size_t cols) {
            std::vector<double> t(a.size());
            for (size_t r = 0; r < rows; ++r)
                for (size_t c = 0; c < cols; ++c) t[c * rows + r] = a[r * cols + c];
            return t;
        };
        const size_t Zh = p.zHalf, Nj = p.Nj;
        upT(transpose(p.Ccos, Zh, Nj), &dd.CcosT); upT(transpose(p.Csin, Zh, Nj), &dd.CsinT);
        upT(transpose(p.CcosM, Zh, Nj), &dd.CcosMT); upT(transpose(p.CsinM, Zh, Nj), &dd.CsinMT);
        upT(transpose(p.Fcos, Nj, Zh), &dd.FcosT); upT(transpose(p.Fsin, Nj, Zh), &dd.FsinT);
    }
    if ((precision == WV_PRECISION_MIXED || precision == WV_PRECISION_FP32X2) && e == cudaSuccess) {
        const std::vector<double> proj64 = mixed_flux_projection(d);
        const std::vector<float> proj = precision == WV_PRECISION_MIXED ? cast<float>(proj64) : to_pairs(proj64);
        const float* q = nullptr;
        e = upload(h, proj, &q);
        dd.fProj = q;
    }
    if (e == cudaSuccess) {
        unsigned* st = nullptr;
        e = alloc(h, sizeof(unsigned), reinterpret_cast<void**>(&st));
        if (e == cudaSuccess) e = cudaMemset(st, 0, sizeof(unsigned));
        dd.status = st;
    }
    if (precision == WV_PRECISION_MIXED && e == cudaSuccess) {
        // tensor-core vertical transform: four accumulators of N <= 128 columns
        const int NP = static_cast<int>((p.zHalf + 15) / 16 * 16);
        const int KE = static_cast<int>(((p.Nj + 1) / 2 + 15) / 16 * 16), KO = static_cast<int>((p.Nj / 2 + 15) / 16 * 16);
        const int K = KE + KO;
        const size_t smem = 6 * (256u * K) + 3 * static_cast<size_t>(NP / 8) * 16u * K;
        if (NP <= 128 && smem <= 220 * 1024) {
            const std::vector<uint16_t> blob = tc_vertical_blob(p, NP, KE, K);
            const uint16_t* q = nullptr;
            e = upload(h, blob, &q);
            dd.tcB = reinterpret_cast<const unsigned short*>(q);
            dd.tcN = NP; dd.tcKE = KE; dd.tcK = K;
            h->tcSmem = smem;
            if (e == cudaSuccess) e = raise_smem_limit(dev::k_vinv_tc, static_cast<int>(smem));
            h->tcAvailable = e == cudaSuccess;
        }
        // forward transform: four accumulators of NF <= 128 output rows over K = zHalf
        const int NF = static_cast<int>(((p.Nj + 1) / 2 + 15) / 16 * 16), KF = static_cast<int>((p.zHalf + 15) / 16 * 16);
        const size_t smemF = 6 * (256u * KF) + 6 * static_cast<size_t>(NF / 8) * 16u * KF;
        if (e == cudaSuccess && h->tcAvailable && NF <= 128 && smemF <= 220 * 1024) {
            const std::vector<uint16_t> blob = tc_forward_blob(p, NF, KF);
            const uint16_t* q = nullptr;
            e = upload(h, blob, &q);
            dd.tcFB = reinterpret_cast<const unsigned short*>(q);
            dd.tcFN = NF; dd.tcFK = KF;
            h->tcFwdSmem = smemF;
            if (e == cudaSuccess) e = raise_smem_limit(dev::k_vfwd_tc, static_cast<int>(smemF));
            h->tcFwdAvailable = e == cudaSuccess;
        }
    }
    if (precision == WV_PRECISION_FP32X2 && e == cudaSuccess) {
        // digit-sliced tensor-core inverse: 2 parities x 4 accumulators of NP <= 64 columns,
        // the zHalf output rows in passes of NP; pass-1 spectra in the y-spectra scratch
        // (free while the vertical inverse runs)
        const int passes = static_cast<int>((p.zHalf + 63) / 64);
        const int NP = static_cast<int>(((p.zHalf + passes - 1) / passes + 15) / 16 * 16);
        const int KH = static_cast<int>(((p.Nj + 1) / 2 + 15) / 16 * 16);
        // A slices + two matrix-block buffers (even and odd j)
        const size_t smem = dev::kTcxDigits * (256u * 2 * KH) + 2 * dev::kTcxDigits * static_cast<size_t>(NP / 8) * 16u * KH;
        const size_t scratchBytes = static_cast<size_t>((p.Nkl + dev::kTcModes - 1) / dev::kTcModes) * dev::kTcModes * p.Nj * 64;
        const size_t yBytes = scratch_sizes(p).y * 2 * elem_size(precision);
        if (8 * NP <= 512 && passes <= 8 && smem <= 220 * 1024 && scratchBytes <= yBytes) {
            const DigitBlob db = tc_digit_blob(p, NP, KH, passes);
            const uint16_t* q = nullptr;
            e = upload(h, db.blob, &q);
            dd.tcxB = reinterpret_cast<const unsigned short*>(q);
            const int32_t* fq = nullptr;
            if (e == cudaSuccess) e = upload(h, db.F, &fq);
            dd.tcxF = fq;
            const std::vector<float> mPairs = to_pairs(d.m);
            const float* mq = nullptr;
            if (e == cudaSuccess) e = upload(h, mPairs, &mq);
            dd.tcxM = mq;
            dd.tcxN = NP; dd.tcxKH = KH; dd.tcxPasses = passes;
            h->tcxSmem = smem;
            if (e == cudaSuccess) e = raise_smem_limit(dev::k_vinv_tcx, static_cast<int>(smem));
            h->tcAvailable = e == cudaSuccess;
        }
    }
    {
        // Default kernels of the flux's vertical transforms, the measured fastest.
        // FP64 and FP32X2: FFTs of the even / odd extension (the reference's own
        // route; fewer operations than the dense contraction, which they beat at
        // every grid) wherever 3 <= Nz <= 513, else the tensor-core inverse of
        // FP32X2 (digit slices) where its blocks fill the GPU, else the dense
        // contraction.  Mixed (FP32 lines are cheap, and the dense contraction's
        // cost per output grows only with Nj): the inverse as FFTs from Nz = 97
        // (warp-register lines: 0.118 ms against 0.125 on the tensor cores and
        // 0.143 dense at 256x256x129, 0.058 against 0.067 and 0.078 at
        // 192x192x97), dense below (0.025 against 0.027 FFT at 128x128x65); the
        // forward transform as FFTs from Nz = 65 (0.078 ms against 0.135 on the
        // tensor cores at 256x256x129, 0.018 against 0.034 dense at 128x128x65),
        // dense below.  The tensor-core kernels stay selectable.
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
        const bool tcFills = h->tcAvailable && static_cast<int>((p.Nkl + dev::kTcModes - 1) / dev::kTcModes) >= sms;
        const bool fft = p.fz.N > 0;
        if (precision == WV_PRECISION_MIXED) {
            h->vinvKind = (fft && p.Nz >= 97) ? WV_VERTICAL_FFT : WV_VERTICAL_CUDA_CORES;
            h->vfwdKind = (fft && p.Nz >= 65) ? WV_VERTICAL_FFT : WV_VERTICAL_CUDA_CORES;
        } else {
            h->vinvKind = fft ? WV_VERTICAL_FFT : tcFills ? WV_VERTICAL_TENSOR_CORES : WV_VERTICAL_CUDA_CORES;
            h->vfwdKind = fft ? WV_VERTICAL_FFT : WV_VERTICAL_CUDA_CORES;
        }
    }
    const auto ss = scratch_sizes(p);
    const size_t cb = 2 * elem_size(precision);
    const size_t R = p.Nx * p.Ny * p.Nz;
    const size_t B = static_cast<size_t>(members);
    if (e == cudaSuccess) e = alloc(h, B * ss.z * cb, &h->zspec);
    if (e == cudaSuccess) e = alloc(h, B * ss.y * cb, &h->yspec);
    if (e == cudaSuccess) e = alloc(h, B * ss.p * cb, &h->pspec);
    if (e == cudaSuccess) e = alloc(h, B * ss.f * cb, &h->fspec);
    void* tmp = nullptr;
    if (e == cudaSuccess) { e = alloc(h, B * sizeof(unsigned long long), &tmp); h->maxSpeed = static_cast<unsigned long long*>(tmp); }
    const size_t stateBytes = B * 6 * p.M * sizeof(double);
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->state = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->flux = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->stage = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->kbuf = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, stateBytes, &tmp); h->acc = static_cast<double*>(tmp); }
    if (e == cudaSuccess) { e = alloc(h, 4 * R * sizeof(double), &tmp); h->fields = static_cast<double*>(tmp); }
    if (e == cudaSuccess)
        e = precision == WV_PRECISION_FP64 ? set_smem_limits<double>(p)
            : precision == WV_PRECISION_MIXED ? set_smem_limits<float>(p) : set_smem_limits<dev::ff>(p);
    if (e == cudaSuccess)
        e = precision == WV_PRECISION_FP64 ? set_smem_limits_w<double>(p)
            : precision == WV_PRECISION_MIXED ? set_smem_limits_w<float>(p) : set_smem_limits_w<dev::ff>(p);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_PLAN_FAILURE;
        cudaGetLastError();  // a failed attribute or allocation call must not surface in a later launch check
        wv_destroy(h);
        return code;
    }
    h->metrics.device_bytes = h->deviceBytes;
    *out = h;
    return WV_SUCCESS;
}

int wv_create(const wv_config* config, int precision, wv_handle** out) { return create_handle(config, precision, 1, out); }

const char* wv_last_message(const wv_handle* h) { return h ? h->message.c_str() : "null handle"; }

int wv_get_sizes(const wv_handle* h, wv_sizes* s) {
    if (!h || !s) return WV_INVALID_POINTER;
    const Plan& p = h->plan;
    s->Nx = p.Nx; s->Ny = p.Ny; s->Nz = p.Nz; s->Nj = p.Nj; s->Nkl = p.Nkl; s->NxHalf = p.NxHalf; s->M = p.M;
    s->active_rows = p.positions; s->kx_columns = p.kxColumns; s->device_bytes = h->deviceBytes;
    return WV_SUCCESS;
}

int wv_get_metrics(const wv_handle* h, wv_metrics* m) {
    if (!h || !m) return WV_INVALID_POINTER;
    *m = h->metrics;
    return WV_SUCCESS;
}

int wv_set_vertical_kernels(wv_handle* h, int inverse_kind, int forward_kind) {
    if (!h) return WV_INVALID_POINTER;
    auto known = [](int k) { return k == WV_VERTICAL_CUDA_CORES || k == WV_VERTICAL_TENSOR_CORES || k == WV_VERTICAL_FFT; };
    if (!known(inverse_kind) || !known(forward_kind))
        return fail(h, WV_INVALID_CONFIGURATION, "Unknown vertical-transform kernel.");
    if ((inverse_kind == WV_VERTICAL_FFT || forward_kind == WV_VERTICAL_FFT) && h->plan.fz.N == 0)
        return fail(h, WV_UNSUPPORTED_OPERATION, "The FFT vertical transform needs 3 <= Nz <= 513.");
    if (inverse_kind == WV_VERTICAL_TENSOR_CORES && !h->tcAvailable)
        return fail(h, WV_UNSUPPORTED_OPERATION,
                    "The tensor-core vertical transform needs a mixed-precision (Nz <= 255) or FP32X2 (Nj <= 96) handle.");
    if (forward_kind == WV_VERTICAL_TENSOR_CORES && !h->tcFwdAvailable)
        return fail(h, WV_UNSUPPORTED_OPERATION,
                    "The tensor-core forward vertical transform needs a mixed-precision handle with Nz <= 255.");
    h->vinvKind = inverse_kind;
    h->vfwdKind = forward_kind;
    return WV_SUCCESS;
}

int wv_set_vertical_kernel(wv_handle* h, int kind) {
    if (!h) return WV_INVALID_POINTER;
    // where only the inverse has a tensor-core kernel (FP32X2 handles), the forward
    // transform keeps the dense contraction
    const int fwd = kind == WV_VERTICAL_TENSOR_CORES && !h->tcFwdAvailable ? WV_VERTICAL_CUDA_CORES : kind;
    return wv_set_vertical_kernels(h, kind, fwd);
}

int wv_get_vertical_kernels(const wv_handle* h, int* inverse_kind, int* forward_kind) {
    if (!h || !inverse_kind || !forward_kind) return WV_INVALID_POINTER;
    *inverse_kind = h->vinvKind;
    *forward_kind = h->vfwdKind;
    return WV_SUCCESS;
}

int wv_get_vertical_kernel(const wv_handle* h, int* kind) {
    if (!h || !kind) return WV_INVALID_POINTER;
    *kind = h->vinvKind;
    return WV_SUCCESS;
}

int wv_set_fft_variants(wv_handle* h, int y_variant, int x_variant) {
    if (!h) return WV_INVALID_POINTER;
    auto known = [](int v) { return v == WV_FFT_REGISTER || v == WV_FFT_STOCKHAM; };
    if (!known(y_variant) || !known(x_variant)) return fail(h, WV_INVALID_CONFIGURATION, "Unknown FFT variant.");
    h->plan.stockhamY = y_variant == WV_FFT_STOCKHAM;
    h->plan.stockhamX = x_variant == WV_FFT_STOCKHAM;
    return WV_SUCCESS;
}

int wv_get_fft_variants(const wv_handle* h, int* y_variant, int* x_variant) {
    if (!h || !y_variant || !x_variant) return WV_INVALID_POINTER;
    const Plan& p = h->plan;
    const bool wy = h->precision == WV_PRECISION_FP64 ? false
                    : h->precision == WV_PRECISION_MIXED ? warp_ry<float>(p) != 0 : warp_ry<dev::ff>(p) != 0;
    const bool wx = h->precision == WV_PRECISION_FP64 ? false
                    : h->precision == WV_PRECISION_MIXED ? warp_rx<float>(p) != 0 : warp_rx<dev::ff>(p) != 0;
    *y_variant = wy ? WV_FFT_REGISTER : WV_FFT_STOCKHAM;
    *x_variant = wx ? WV_FFT_REGISTER : WV_FFT_STOCKHAM;
    return WV_SUCCESS;
}

int wv_get_device_status(wv_handle* h, unsigned* status) {
    if (!h || !status) return WV_INVALID_POINTER;
    cudaSetDevice(h->device);
    const cudaError_t e = cudaMemcpy(status, h->dd.status, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return finish(h, e, "device status");
}

int wv_error_tolerances(wv_handle* h, double absolute_tolerance_scale, double* wave, double* vortex) {
    if (!h) return WV_INVALID_POINTER;
    if (!wave || !vortex) return fail(h, WV_INVALID_POINTER, "Tolerance outputs must be nonnull.");
    std::vector<double> w, v;
    const Status st = wvgpu::adaptive_error_tolerances(h->desc, absolute_tolerance_scale, w, v);
    if (!st) return fail(h, st.code, st.message);
    std::memcpy(wave, w.data(), w.size() * sizeof(double));
    std::memcpy(vortex, v.data(), v.size() * sizeof(double));
    return WV_SUCCESS;
}

int wv_reset_device_status(wv_handle* h) {
    if (!h) return WV_INVALID_POINTER;
    cudaSetDevice(h->device);
    return finish(h, cudaMemset(h->dd.status, 0, sizeof(unsigned)), "device status");
}

// ---- test hooks ----------------------------------------------------------------------
// Failure injection on the host (and one bounded in-kernel wait made to run
// out): how the contract tests reach the error paths without a GPU fault.

int wv_test_fail_allocation_after(long long n) {
    g_failAllocationAfter.store(n < 0 ? -1 : n);
    return WV_SUCCESS;
}

long long wv_test_live_device_bytes(void) { return g_liveDeviceBytes.load(); }

int wv_test_fail_launch_after(wv_handle* h, long long n) {
    if (!h) return WV_INVALID_POINTER;
    h->failLaunchAfter = n < 0 ? -1 : n;
    h->injectedFailure = false;
    return WV_SUCCESS;
}

int wv_test_hold_busy(wv_handle* h, int hold) {
    if (!h) return WV_INVALID_POINTER;
    h->busy.store(hold != 0);
    return WV_SUCCESS;
}

int wv_test_inject_wait_timeout(wv_handle* h, unsigned polls) {
    if (!h) return WV_INVALID_POINTER;
    h->dd.injectWaitPolls = polls;
    return WV_SUCCESS;
}

int wv_set_stage_instrumentation(wv_handle* h, int enabled) {
    if (!h) return WV_INVALID_POINTER;
    if (enabled) {
        cudaSetDevice(h->device);
        for (auto& ev : h->ev) {
            if (!ev) {
                const cudaError_t e = cudaEventCreate(&ev);
                if (e != cudaSuccess) return cuda_fail(h, e, "stage instrumentation");
            }
        }
        h->stages = wv_stage_times{};
    }
    h->instrument = enabled != 0;
    return WV_SUCCESS;
}

int wv_get_stage_times(const wv_handle* h, wv_stage_times* t) {
    if (!h || !t) return WV_INVALID_POINTER;
    *t = h->stages;
    return WV_SUCCESS;
}

int wv_set_forcing(wv_handle* h, uint32_t flags) {
    if (!h) return WV_INVALID_POINTER;
    if (!(flags & WV_FORCING_NONLINEAR_ADVECTION) || (flags & ~3u))
        return fail(h, WV_UNSUPPORTED_OPERATION, "Supported schedules: nonlinear advection, optionally with adaptive damping.");
    if ((flags & WV_FORCING_ADAPTIVE_DAMPING) && !h->hasDamping)
        return fail(h, WV_UNSUPPORTED_OPERATION, "Adaptive damping requires nonzero Coriolis frequency.");
    h->forcing = flags;
    return WV_SUCCESS;
}

// ---- device-pointer entries --------------------------------------------------------

int wv_nonlinear_flux_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                             double* Fp, double* Fm, double* F0, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e = flux_any(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, static_cast<cudaStream_t>(stream));
    h->metrics.nonlinear_flux_calls++;
    return finish(h, e, "nonlinear flux");
}

int wv_evaluate_rhs_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                           double* Fp, double* Fm, double* F0, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const bool damping = (h->forcing & WV_FORCING_ADAPTIVE_DAMPING) != 0;
    const cudaError_t e = flux_any(h, t, t0, Ap, Am, A0, Fp, Fm, F0, damping, static_cast<cudaStream_t>(stream));
    h->metrics.rhs_evaluations++;
    return finish(h, e, "right-hand side");
}

int wv_inverse_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* fields,
                      void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Inverse transform received a null pointer.");
    const size_t fb = 4 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    for (const void* in : {static_cast<const void*>(Ap), static_cast<const void*>(Am), static_cast<const void*>(A0)})
        if (overlaps(fields, fb, in, cb)) return fail(h, WV_OVERLAPPING_ARRAYS, "Inverse spatial output must not overlap coefficient inputs.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e = h->precision == WV_PRECISION_FP64
                              ? launch_inverse<double>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream))
                              : h->precision == WV_PRECISION_MIXED ? launch_inverse<float>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream))
                                                                         : launch_inverse<dev::ff>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream));
    h->metrics.inverse_calls++;
    return finish(h, e, "inverse transform");
}

// ---- advection fields (nonlinearFluxWithAdvectionFields / UsingAdvectionFields, kernel.cpp:1148-1171;
//      transformWaveVortexToUVW, kernel.cpp:696-717) ----------------------------------------

static int advection_entry_checks(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                                  double* Fp, double* Fm, double* F0, const double* fields, const char* what) {
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    if (!fields) return fail(h, WV_INVALID_POINTER, std::string(what) + " pointer must be nonnull.");
    if (h->dd.members != 1) return fail(h, WV_UNSUPPORTED_OPERATION, "Advection fields are per single-state handle.");
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    for (const void* p : {static_cast<const void*>(Ap), static_cast<const void*>(Am), static_cast<const void*>(A0),
                          static_cast<const void*>(Fp), static_cast<const void*>(Fm), static_cast<const void*>(F0)})
        if (overlaps(fields, fb, p, cb))
            return fail(h, WV_OVERLAPPING_ARRAYS, std::string(what) + " must not overlap the state or flux arrays.");
    return WV_SUCCESS;
}

int wv_nonlinear_flux_with_advection_fields_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am,
                                                   const double* A0, double* Fp, double* Fm, double* F0, double* fields,
                                                   void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = advection_entry_checks(h, t, t0, Ap, Am, A0, Fp, Fm, F0, fields, "Advection fields"); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e = flux_any(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, static_cast<cudaStream_t>(stream), nullptr, fields);
    h->metrics.nonlinear_flux_calls++;
    return finish(h, e, "nonlinear flux");
}

int wv_nonlinear_flux_using_advection_fields_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am,
                                                    const double* A0, double* Fp, double* Fm, double* F0,
                                                    const double* fields, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = advection_entry_checks(h, t, t0, Ap, Am, A0, Fp, Fm, F0, fields, "Prepared advection fields"); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e =
        flux_any(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, static_cast<cudaStream_t>(stream), nullptr, nullptr, fields);
    h->metrics.nonlinear_flux_calls++;
    return finish(h, e, "nonlinear flux");
}

int wv_inverse_uvw_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                          double* fields, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Inverse transform received a null pointer.");
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    for (const void* in : {static_cast<const void*>(Ap), static_cast<const void*>(Am), static_cast<const void*>(A0)})
        if (overlaps(fields, fb, in, cb)) return fail(h, WV_OVERLAPPING_ARRAYS, "Inverse spatial output must not overlap coefficient inputs.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e = h->precision == WV_PRECISION_FP64
                              ? launch_inverse<double>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream), 3)
                              : h->precision == WV_PRECISION_MIXED ? launch_inverse<float>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream), 3)
                                                                         : launch_inverse<dev::ff>(h, t, t0, Ap, Am, A0, fields, static_cast<cudaStream_t>(stream), 3);
    h->metrics.inverse_calls++;
    return finish(h, e, "inverse transform");
}

// Host-pointer forms: state, flux and fields through the handle's device mirrors.
static int host_advection_flux(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                               double* Fp, double* Fm, double* F0, double* fieldsOut, const double* fieldsIn) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !Fp || !Fm || !F0 || !(fieldsOut || fieldsIn))
        return fail(h, WV_INVALID_POINTER, "Nonlinear flux received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && fieldsIn) e = cudaMemcpyAsync(h->fields, fieldsIn, fb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = flux_any(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->flux, h->flux + M2, h->flux + 2 * M2, false, s,
                     nullptr, fieldsOut ? h->fields : nullptr, fieldsIn ? h->fields : nullptr);
    double* out[] = {Fp, Fm, F0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(out[c], reinterpret_cast<char*>(h->flux) + c * cb, cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && fieldsOut) e = cudaMemcpyAsync(fieldsOut, h->fields, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    h->metrics.nonlinear_flux_calls++;
    return finish(h, e, "nonlinear flux");
}

int wv_nonlinear_flux_with_advection_fields(wv_handle* h, double t, double t0, const double* Ap, const double* Am,
                                            const double* A0, double* Fp, double* Fm, double* F0, double* fields) {
    return host_advection_flux(h, t, t0, Ap, Am, A0, Fp, Fm, F0, fields, nullptr);
}

int wv_nonlinear_flux_using_advection_fields(wv_handle* h, double t, double t0, const double* Ap, const double* Am,
                                             const double* A0, double* Fp, double* Fm, double* F0, const double* fields) {
    return host_advection_flux(h, t, t0, Ap, Am, A0, Fp, Fm, F0, nullptr, fields);
}

int wv_inverse_uvw(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* fields) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Inverse transform received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64
                ? launch_inverse<double>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s, 3)
                : h->precision == WV_PRECISION_MIXED ? launch_inverse<float>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s, 3)
                                                           : launch_inverse<dev::ff>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s, 3);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fields, h->fields, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    h->metrics.inverse_calls++;
    return finish(h, e, "inverse transform");
}

int wv_field_derivatives_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                                int field, double* out, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (field < 0 || field > 3) return fail(h, WV_INVALID_CONFIGURATION, "Unknown dynamical field derivative target.");
    if (!Ap || !Am || !A0 || !out) return fail(h, WV_INVALID_POINTER, "Field derivatives received a null pointer.");
    if (h->dd.members != 1) return fail(h, WV_UNSUPPORTED_OPERATION, "Field derivatives are per single-state handle.");
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    for (const void* in : {static_cast<const void*>(Ap), static_cast<const void*>(Am), static_cast<const void*>(A0)})
        if (overlaps(out, fb, in, cb)) return fail(h, WV_OVERLAPPING_ARRAYS, "Field derivatives must not overlap coefficient inputs.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    auto s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = h->precision == WV_PRECISION_FP64 ? launch_field_derivatives<double>(h, t, t0, Ap, Am, A0, field, out, s)
                : h->precision == WV_PRECISION_MIXED ? launch_field_derivatives<float>(h, t, t0, Ap, Am, A0, field, out, s)
                                                     : launch_field_derivatives<dev::ff>(h, t, t0, Ap, Am, A0, field, out, s);
    return finish(h, e, "field derivatives");
}

int wv_family_derivatives_device(wv_handle* h, int ffamily, const double* Apm, const double* A0, double* fields,
                                 void* stream) {
    if (!h) return WV_INVALID_POINTER;
    if (!Apm || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Field-family derivatives received a null pointer.");
    if (h->dd.members != 1) return fail(h, WV_UNSUPPORTED_OPERATION, "Field-family derivatives are per single-state handle.");
    const size_t fb = 4 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    if (overlaps(fields, fb, Apm, cb) || overlaps(fields, fb, A0, cb))
        return fail(h, WV_OVERLAPPING_ARRAYS, "Field derivative output must not overlap coefficient inputs.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    auto s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = h->precision == WV_PRECISION_FP64 ? launch_family_derivatives<double>(h, ffamily != 0, Apm, A0, fields, s)
                : h->precision == WV_PRECISION_MIXED ? launch_family_derivatives<float>(h, ffamily != 0, Apm, A0, fields, s)
                                                     : launch_family_derivatives<dev::ff>(h, ffamily != 0, Apm, A0, fields, s);
    return finish(h, e, "field-family derivatives");
}

int wv_family_derivatives(wv_handle* h, int ffamily, const double* Apm, const double* A0, double* fields) {
    if (!h) return WV_INVALID_POINTER;
    if (!Apm || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Field-family derivatives received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = 4 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaMemcpyAsync(h->state, Apm, cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->state + M2, A0, cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64 ? launch_family_derivatives<double>(h, ffamily != 0, h->state, h->state + M2, h->fields, s)
                : h->precision == WV_PRECISION_MIXED ? launch_family_derivatives<float>(h, ffamily != 0, h->state, h->state + M2, h->fields, s)
                                                     : launch_family_derivatives<dev::ff>(h, ffamily != 0, h->state, h->state + M2, h->fields, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fields, h->fields, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return finish(h, e, "field-family derivatives");
}

static int scalar_entry_checks(wv_handle* h, const double* scalar, const double* fields, const double* rhs) {
    if (!scalar || !rhs) return fail(h, WV_INVALID_POINTER, "F-grid scalar input and output pointers must be nonnull.");
    if (!fields) return fail(h, WV_INVALID_POINTER, "Advection fields pointer must be nonnull.");
    if (h->dd.members != 1) return fail(h, WV_UNSUPPORTED_OPERATION, "Scalar advection is per single-state handle.");
    const size_t bytes = h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    if (overlaps(scalar, bytes, rhs, bytes) || overlaps(fields, 3 * bytes, scalar, bytes) || overlaps(fields, 3 * bytes, rhs, bytes))
        return fail(h, WV_OVERLAPPING_ARRAYS, "Tracer scalar, velocity, and RHS arrays must not overlap.");
    return WV_SUCCESS;
}

int wv_advect_fgrid_scalar_device(wv_handle* h, const double* scalar, const double* fields, int antialias, double* rhs,
                                  void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = scalar_entry_checks(h, scalar, fields, rhs); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    rc = ensure_scalar(h); if (rc) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = h->precision == WV_PRECISION_FP64 ? launch_scalar_advection<double>(h, scalar, fields, antialias != 0, rhs, s)
                : h->precision == WV_PRECISION_MIXED ? launch_scalar_advection<float>(h, scalar, fields, antialias != 0, rhs, s)
                                                     : launch_scalar_advection<dev::ff>(h, scalar, fields, antialias != 0, rhs, s);
    return finish(h, e, "scalar advection");
}

int wv_advect_fgrid_scalar(wv_handle* h, const double* scalar, const double* fields, int antialias, double* rhs) {
    if (!h) return WV_INVALID_POINTER;
    int rc = scalar_entry_checks(h, scalar, fields, rhs); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    rc = ensure_scalar(h); if (rc) return rc;
    const size_t R = h->plan.Nx * h->plan.Ny * h->plan.Nz, bytes = R * sizeof(double);
    auto s = h->stream;
    // h->fields holds 4 R doubles: the scalar in the first R, (u, v, w) in the next 3 R
    double* dScalar = h->fields;
    double* dAdv = h->fields + R;
    double* dRhs = h->scalarRhs;
    cudaError_t e = cudaMemcpyAsync(dScalar, scalar, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dAdv, fields, 3 * bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64 ? launch_scalar_advection<double>(h, dScalar, dAdv, antialias != 0, dRhs, s)
                : h->precision == WV_PRECISION_MIXED ? launch_scalar_advection<float>(h, dScalar, dAdv, antialias != 0, dRhs, s)
                                                     : launch_scalar_advection<dev::ff>(h, dScalar, dAdv, antialias != 0, dRhs, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rhs, dRhs, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return finish(h, e, "scalar advection");
}

int wv_field_derivatives(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, int field,
                         double* out) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (field < 0 || field > 3) return fail(h, WV_INVALID_CONFIGURATION, "Unknown dynamical field derivative target.");
    if (!Ap || !Am || !A0 || !out) return fail(h, WV_INVALID_POINTER, "Field derivatives received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = 3 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64 ? launch_field_derivatives<double>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, field, h->fields, s)
                : h->precision == WV_PRECISION_MIXED ? launch_field_derivatives<float>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, field, h->fields, s)
                                                     : launch_field_derivatives<dev::ff>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, field, h->fields, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, h->fields, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return finish(h, e, "field derivatives");
}

int wv_forward_device(wv_handle* h, const double* fields, double t, double t0, double* Ap, double* Am, double* A0, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Forward transform received a null pointer.");
    const int nch = h->desc.c.is_hydrostatic ? 3 : 4;
    const size_t fb = nch * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double), cb = h->plan.M * 16;
    const void* outs[] = {Ap, Am, A0};
    for (int i = 0; i < 3; ++i) {
        if (overlaps(outs[i], cb, fields, fb)) return fail(h, WV_OVERLAPPING_ARRAYS, "Forward coefficient outputs must not overlap the spatial input.");
        for (int j = i + 1; j < 3; ++j)
            if (overlaps(outs[i], cb, outs[j], cb)) return fail(h, WV_OVERLAPPING_ARRAYS, "Forward coefficient outputs must not overlap each other.");
    }
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const cudaError_t e = h->precision == WV_PRECISION_FP64
                              ? launch_forward<double>(h, fields, t, t0, Ap, Am, A0, static_cast<cudaStream_t>(stream))
                              : h->precision == WV_PRECISION_MIXED ? launch_forward<float>(h, fields, t, t0, Ap, Am, A0, static_cast<cudaStream_t>(stream))
                                                                         : launch_forward<dev::ff>(h, fields, t, t0, Ap, Am, A0, static_cast<cudaStream_t>(stream));
    h->metrics.forward_calls++;
    return finish(h, e, "forward transform");
}

int wv_rk4_steps_device(wv_handle* h, double* Ap, double* Am, double* A0, double* t, double t0, double dt, int n, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    if (!Ap || !Am || !A0 || !t) return fail(h, WV_INVALID_POINTER, "RK4 received a null pointer.");
    int rc = check_times(h, *t, t0); if (rc) return rc;
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    if (n < 0) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step count must be nonnegative.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    cudaSetDevice(h->device);
    auto s = static_cast<cudaStream_t>(stream);
    const size_t cb = h->plan.M * 16;
    cudaError_t e = cudaSuccess;
    const double* src[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, src[c], cb, cudaMemcpyDeviceToDevice, s);
    double tt = *t;
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
        e = rk4_step(h, tt, t0, dt, s);
        if (e == cudaSuccess && h->rk4Dense) { h->denseValid = true; h->denseTi = tt; h->denseTf = tt + dt; }
        tt = tt + dt;
    }
    double* dst[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(dst[c], reinterpret_cast<char*>(h->state) + c * cb, cb, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "RK4");
    *t = tt;
    return WV_SUCCESS;
}

// WVFixedStepRK4Options::retainDenseOutput (PortableRuntime/include/WaveVortexRuntime/
// WVRungeKutta.hpp:52-54): keeps the last step's end states and first and
// fourth stage derivatives on the device (4 state-sized buffers, allocated on
// first use) for wv_rk4_dense_output_device.
int wv_rk4_set_dense_output(wv_handle* h, int enabled) {
    if (!h) return WV_INVALID_POINTER;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    if (enabled && !h->denseBuf) {
        cudaSetDevice(h->device);
        void* p = nullptr;
        const cudaError_t e = alloc(h, 4 * 6 * h->plan.M * h->dd.members * sizeof(double), &p);
        if (e != cudaSuccess) return cuda_fail(h, e, "RK4 dense-output buffers");
        h->denseBuf = static_cast<double*>(p);
    }
    h->rk4Dense = enabled != 0;
    h->denseValid = false;
    return WV_SUCCESS;
}

// WVFixedStepRK4::advanceToTime (PortableRuntime/src/WVRungeKutta.cpp:464-480):
// steps of min(dt, final_time - t) until final_time; *t ends at final_time.
int wv_rk4_advance_to_time_device(wv_handle* h, double* Ap, double* Am, double* A0, double* t, double t0,
                                  double final_time, double dt, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    if (!Ap || !Am || !A0 || !t) return fail(h, WV_INVALID_POINTER, "RK4 received a null pointer.");
    int rc = check_times(h, *t, t0); if (rc) return rc;
    if (final_time < *t || !std::isfinite(final_time))
        return fail(h, WV_INVALID_CONFIGURATION, "RK4 cannot advance backward or to a nonfinite time.");
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    cudaSetDevice(h->device);
    auto s = static_cast<cudaStream_t>(stream);
    const size_t cb = h->plan.M * 16;
    cudaError_t e = cudaSuccess;
    const double* src[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, src[c], cb, cudaMemcpyDeviceToDevice, s);
    double tt = *t;
    while (tt < final_time && e == cudaSuccess) {
        const double step = std::min(dt, final_time - tt);
        if (!(step > 0.0)) break;
        e = rk4_step(h, tt, t0, step, s);
        if (e == cudaSuccess && h->rk4Dense) { h->denseValid = true; h->denseTi = tt; h->denseTf = tt + step; }
        tt = tt + step;
    }
    double* dst[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(dst[c], reinterpret_cast<char*>(h->state) + c * cb, cb, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "RK4");
    *t = final_time;
    return WV_SUCCESS;
}

// WVFixedStepRK4::evaluateDenseOutput (WVRungeKutta.cpp:482-541): the cubic
// Hermite interpolant of the last step through its end states, with the first
// and fourth stage derivatives as end slopes.
int wv_rk4_dense_output_device(wv_handle* h, double time, double* Ap, double* Am, double* A0, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    if (!Ap || !Am || !A0) return fail(h, WV_INVALID_POINTER, "Dense output received a null pointer.");
    if (!h->rk4Dense || !h->denseValid) return fail(h, WV_UNSUPPORTED_OPERATION, "RK4 dense output is unavailable.");
    const double tol = 8.0 * std::numeric_limits<double>::epsilon() *
                       std::max({1.0, std::abs(h->denseTi), std::abs(h->denseTf)});
    if (time < h->denseTi - tol || time > h->denseTf + tol)
        return fail(h, WV_INVALID_CONFIGURATION, "Dense-output time is outside the accepted interval.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 dense-output evaluation is not reentrant.");
    cudaSetDevice(h->device);
    const double hstep = h->denseTf - h->denseTi;
    double theta = hstep == 0.0 ? 0.0 : (time - h->denseTi) / hstep;
    theta = std::max(0.0, std::min(1.0, theta));
    const double t2 = theta * theta, t3 = t2 * theta, ew = 3 * t2 - 2 * t3, iw = 1 - ew,
                 isw = hstep * (theta - 2 * t2 + t3), esw = hstep * (t3 - t2);
    const size_t n = 6 * h->plan.M, M2 = 2 * h->plan.M;
    const unsigned grid = static_cast<unsigned>(std::min<size_t>((M2 + 255) / 256, wvgpu::grid_cap(16)));
    const double* b = h->denseBuf;
    dev::k_rk4_dense<<<dim3(grid, 3), 256, 0, static_cast<cudaStream_t>(stream)>>>(b, b + n, b + 2 * n, b + 3 * n, iw, ew, isw,
                                                                                   esw, Ap, Am, A0, M2);
    h->metrics.kernel_launches += 1;
    return finish(h, cudaGetLastError(), "RK4 dense output");
}

int wv_rk4_advance_to_time(wv_handle* h, double* Ap, double* Am, double* A0, double* t, double t0, double final_time,
                           double dt) {
    if (!h) return WV_INVALID_POINTER;
    if (!Ap || !Am || !A0 || !t) return fail(h, WV_INVALID_POINTER, "RK4 received a null pointer.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16;
    auto s = h->stream;
    double* hostPtr[] = {Ap, Am, A0};
    double* devPtr[] = {h->flux, h->flux + 2 * h->plan.M, h->flux + 4 * h->plan.M};
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) e = cudaMemcpyAsync(devPtr[c], hostPtr[c], cb, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(h, e, "RK4 state upload");
    const int rc = wv_rk4_advance_to_time_device(h, devPtr[0], devPtr[1], devPtr[2], t, t0, final_time, dt, s);
    if (rc) return rc;
    for (int c = 0; c < 3 && e == cudaSuccess; ++c) e = cudaMemcpyAsync(hostPtr[c], devPtr[c], cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return finish(h, e, "RK4 state download");
}

// ---- host-pointer entries ------------------------------------------------------------

static int host_flux(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* Fp,
                     double* Fm, double* F0, bool scheduled) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16;
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    const size_t M2 = 2 * h->plan.M;
    const bool damping = scheduled && (h->forcing & WV_FORCING_ADAPTIVE_DAMPING);
    if (e == cudaSuccess)
        e = flux_any(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->flux, h->flux + M2, h->flux + 2 * M2, damping, s);
    double* out[] = {Fp, Fm, F0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(out[c], reinterpret_cast<char*>(h->flux) + c * cb, cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (scheduled) h->metrics.rhs_evaluations++; else h->metrics.nonlinear_flux_calls++;
    return finish(h, e, scheduled ? "right-hand side" : "nonlinear flux");
}

int wv_nonlinear_flux(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* Fp,
                      double* Fm, double* F0) {
    return host_flux(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false);
}

int wv_evaluate_rhs(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* Fp,
                    double* Fm, double* F0) {
    return host_flux(h, t, t0, Ap, Am, A0, Fp, Fm, F0, true);
}

int wv_inverse(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0, double* fields) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Inverse transform received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = 4 * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64
                ? launch_inverse<double>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s)
                : h->precision == WV_PRECISION_MIXED ? launch_inverse<float>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s)
                                                           : launch_inverse<dev::ff>(h, t, t0, h->state, h->state + M2, h->state + 2 * M2, h->fields, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fields, h->fields, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    h->metrics.inverse_calls++;
    return finish(h, e, "inverse transform");
}

int wv_forward(wv_handle* h, const double* fields, double t, double t0, double* Ap, double* Am, double* A0) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !fields) return fail(h, WV_INVALID_POINTER, "Forward transform received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    const int nch = h->desc.c.is_hydrostatic ? 3 : 4;
    const size_t cb = h->plan.M * 16, M2 = 2 * h->plan.M;
    const size_t fb = nch * h->plan.Nx * h->plan.Ny * h->plan.Nz * sizeof(double);
    auto s = h->stream;
    cudaError_t e = cudaMemcpyAsync(h->fields, fields, fb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = h->precision == WV_PRECISION_FP64
                ? launch_forward<double>(h, h->fields, t, t0, h->flux, h->flux + M2, h->flux + 2 * M2, s)
                : h->precision == WV_PRECISION_MIXED ? launch_forward<float>(h, h->fields, t, t0, h->flux, h->flux + M2, h->flux + 2 * M2, s)
                                                           : launch_forward<dev::ff>(h, h->fields, t, t0, h->flux, h->flux + M2, h->flux + 2 * M2, s);
    double* out[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(out[c], reinterpret_cast<char*>(h->flux) + c * cb, cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    h->metrics.forward_calls++;
    return finish(h, e, "forward transform");
}

int wv_rk4_steps(wv_handle* h, double* Ap, double* Am, double* A0, double* t, double t0, double dt, int n) {
    if (!h) return WV_INVALID_POINTER;
    if (!Ap || !Am || !A0 || !t) return fail(h, WV_INVALID_POINTER, "RK4 received a null pointer.");
    int rc = check_times(h, *t, t0); if (rc) return rc;
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    if (n < 0) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step count must be nonnegative.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    cudaSetDevice(h->device);
    const size_t cb = h->plan.M * 16;
    auto s = h->stream;
    cudaError_t e = cudaSuccess;
    const double* in[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(h->state) + c * cb, in[c], cb, cudaMemcpyHostToDevice, s);
    double tt = *t;
    for (int i = 0; i < n && e == cudaSuccess; ++i) {
        e = rk4_step(h, tt, t0, dt, s);
        if (e == cudaSuccess && h->rk4Dense) { h->denseValid = true; h->denseTi = tt; h->denseTf = tt + dt; }
        tt = tt + dt;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // A failed step leaves the caller's state untouched (TestWVForcingAndRK4.cpp:316-319).
    double* out[] = {Ap, Am, A0};
    for (int c = 0; c < 3 && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(out[c], reinterpret_cast<char*>(h->state) + c * cb, cb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(h, e, "RK4");
    *t = tt;
    return WV_SUCCESS;
}


// ---- adjoint entry points --------------------------------------------------------------

static int adjoint_preamble(wv_handle* h) {
    if (h->forcing & WV_FORCING_ADAPTIVE_DAMPING)
        return fail(h, WV_UNSUPPORTED_OPERATION, "The adjoint covers the nonlinear advection schedule; disable adaptive damping.");
    cudaSetDevice(h->device);
    return ensure_adjoint(h);
}

int wv_flux_vjp_device(wv_handle* h, double t, double t0, const double* Ap, const double* Am, const double* A0,
                       const double* Fpb, const double* Fmb, const double* F0b, double* Apb, double* Amb, double* A0b,
                       void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    const void* ptrs[] = {Ap, Am, A0, Fpb, Fmb, F0b, Apb, Amb, A0b};
    for (const void* q : ptrs) if (!q) return fail(h, WV_INVALID_POINTER, "Flux VJP received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    rc = adjoint_preamble(h); if (rc) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = h->precision == WV_PRECISION_FP64
        ? launch_flux_vjp<double>(h, t, t0, Ap, Am, A0, Fpb, Fmb, F0b, Apb, Amb, A0b, s)
        : h->precision == WV_PRECISION_MIXED ? launch_flux_vjp<float>(h, t, t0, Ap, Am, A0, Fpb, Fmb, F0b, Apb, Amb, A0b, s)
                                                   : launch_flux_vjp<dev::ff>(h, t, t0, Ap, Am, A0, Fpb, Fmb, F0b, Apb, Amb, A0b, s);
    return finish(h, e, "flux VJP");
}

int wv_inverse_vjp_device(wv_handle* h, double t, double t0, const double* fb, double* Apb, double* Amb, double* A0b,
                          void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!fb || !Apb || !Amb || !A0b) return fail(h, WV_INVALID_POINTER, "Inverse VJP received a null pointer.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaSetDevice(h->device);
    rc = ensure_adjoint(h); if (rc) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = h->precision == WV_PRECISION_FP64    ? launch_inverse_vjp<double>(h, t, t0, fb, Apb, Amb, A0b, s)
                          : h->precision == WV_PRECISION_MIXED ? launch_inverse_vjp<float>(h, t, t0, fb, Apb, Amb, A0b, s)
                                                               : launch_inverse_vjp<dev::ff>(h, t, t0, fb, Apb, Amb, A0b, s);
    return finish(h, e, "inverse VJP");
}

static cudaError_t gather3(wv_handle* h, double* dst, const double* a, const double* b, const double* c, cudaStream_t s) {
    const size_t cb = h->plan.M * 16;
    const double* src[] = {a, b, c};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
        e = cudaMemcpyAsync(reinterpret_cast<char*>(dst) + i * cb, src[i], cb, cudaMemcpyDeviceToDevice, s);
    return e;
}
static cudaError_t scatter3(wv_handle* h, const double* src, double* a, double* b, double* c, cudaStream_t s) {
    const size_t cb = h->plan.M * 16;
    double* dst[] = {a, b, c};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 3 && e == cudaSuccess; ++i)
        e = cudaMemcpyAsync(dst[i], reinterpret_cast<const char*>(src) + i * cb, cb, cudaMemcpyDeviceToDevice, s);
    return e;
}

int wv_rk4_step_vjp_device(wv_handle* h, const double* Ap, const double* Am, const double* A0, double t, double t0, double dt,
                           double* Apb, double* Amb, double* A0b, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !Apb || !Amb || !A0b) return fail(h, WV_INVALID_POINTER, "RK4 VJP received a null pointer.");
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    rc = adjoint_preamble(h); if (rc) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    cudaError_t e = gather3(h, h->state, Ap, Am, A0, s);
    if (e == cudaSuccess) e = gather3(h, h->ybin, Apb, Amb, A0b, s);
    if (e == cudaSuccess) e = rk4_step_vjp(h, h->state, t, t0, dt, h->ybin, s);
    if (e == cudaSuccess) e = scatter3(h, h->ybacc, Apb, Amb, A0b, s);
    return finish(h, e, "RK4 VJP");
}

int wv_rk4_adjoint_device(wv_handle* h, const double* Ap, const double* Am, const double* A0, double t, double t0, double dt,
                          int n, int K, double* Apb, double* Amb, double* A0b, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    if (!Ap || !Am || !A0 || !Apb || !Amb || !A0b) return fail(h, WV_INVALID_POINTER, "RK4 adjoint received a null pointer.");
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(h, WV_INVALID_CONFIGURATION, "RK4 step size must be finite and positive.");
    if (n < 0 || K < 1) return fail(h, WV_INVALID_CONFIGURATION, "Step count must be nonnegative and the checkpoint interval positive.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "RK4 stepping is not reentrant.");
    rc = adjoint_preamble(h); if (rc) return rc;
    auto s = static_cast<cudaStream_t>(stream);
    const size_t stateBytes = 6 * h->plan.M * sizeof(double);
    const int ncp = (n + K - 1) / K;
    cudaError_t e = cudaSuccess;
    void* tmp = nullptr;
    while (static_cast<int>(h->checkpoints.size()) < ncp && e == cudaSuccess) {
        e = alloc(h, stateBytes, &tmp);
        h->checkpoints.push_back(static_cast<double*>(tmp));
    }
    // real rows of the x pass of every stage flux of a segment, in one or (when
    // half the free memory holds them) two segment slots; two slots let the
    // recomputation of the next segment run on a side stream during the
    // backward sweep of the current one
    const size_t yBytes = (3 + 3 * h->plan.targets.count) * h->plan.Nx * h->plan.Ny * h->plan.Nz * elem_size(h->precision);
    int slots = 0;
    if (e == cudaSuccess) {
        size_t freeB = 0, totalB = 0;
        e = cudaMemGetInfo(&freeB, &totalB);
        for (int want = 2; want >= 1 && e == cudaSuccess && slots == 0; --want) {
            const size_t haveY = h->ystore.size(), haveS = h->segment.size();
            const size_t needY = static_cast<size_t>(std::max<int>(0, 4 * K * want - static_cast<int>(haveY))) * yBytes;
            const size_t needS = static_cast<size_t>(std::max<int>(0, 4 * K * want - static_cast<int>(haveS))) * stateBytes;
            if (needY + needS <= freeB / 2) slots = want;
        }
    }
    const int nSlots = std::max(slots, 1);
    while (static_cast<int>(h->segment.size()) < 4 * K * nSlots && e == cudaSuccess) {
        e = alloc(h, stateBytes, &tmp);
        h->segment.push_back(static_cast<double*>(tmp));
    }
    while (slots > 0 && static_cast<int>(h->ystore.size()) < 4 * K * slots && e == cudaSuccess) {
        e = alloc(h, yBytes, &tmp);
        h->ystore.push_back(tmp);
    }
    if (e == cudaSuccess && !h->ybAlt) { e = alloc(h, stateBytes, &tmp); h->ybAlt = static_cast<double*>(tmp); }
    const bool pipelined = slots == 2;
    if (e == cudaSuccess && pipelined && !h->adjStream) {
        e = cudaStreamCreateWithFlags(&h->adjStream, cudaStreamNonBlocking);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
            e = cudaEventCreateWithFlags(&h->slotReady[i], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->slotFree[i], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->fwdDone, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "RK4 adjoint checkpoints");
    h->metrics.device_bytes = h->deviceBytes;
    const bool keepY = slots > 0;
    std::vector<double> times(n + 1);
    times[0] = t;
    for (int i = 0; i < n; ++i) times[i + 1] = times[i] + dt;
    auto slotOf = [&](int seg) { return pipelined ? (seg & 1) : 0; };
    // Stage states (and real rows) of the steps first..last-1 from the state in the
    // slot's first entry, the state of each next step in the following entry;
    // endOut, when given, receives the state after the last step.
    auto record = [&](int first, int last, int slot, cudaStream_t st, double* endOut) {
        cudaError_t r = cudaSuccess;
        for (int i = first; i < last && r == cudaSuccess; ++i) {
            double** q = h->segment.data() + 4 * K * slot + 4 * (i - first);
            void* const* ys = keepY ? h->ystore.data() + 4 * K * slot + 4 * (i - first) : nullptr;
            r = rk4_stages(h, q[0], times[i], t0, dt, q[1], q[2], q[3], i + 1 < last ? q[4] : endOut, st, ys);
        }
        return r;
    };
    // forward pass: checkpoints at the start of each segment; the segments that
    // have a slot of their own from the start -- the last one, and with two slots
    // the one before it -- are recorded directly, so their recomputation is skipped
    const int directSeg = pipelined && ncp >= 2 ? ncp - 2 : -1;
    e = gather3(h, h->state, Ap, Am, A0, s);
    for (int seg = 0; seg < ncp && e == cudaSuccess; ++seg) {
        const int first = seg * K, last = std::min(n, first + K);
        if (seg + 1 < ncp && seg != directSeg) {
            e = cudaMemcpyAsync(h->checkpoints[seg], h->state, stateBytes, cudaMemcpyDeviceToDevice, s);
            for (int i = first; i < last && e == cudaSuccess; ++i) e = rk4_step(h, times[i], t0, dt, s);
        } else {
            // the same stage arithmetic as rk4_step, so the states are those a recomputation gives
            const int sl = slotOf(seg);
            e = cudaMemcpyAsync(h->segment[4 * K * sl], h->state, stateBytes, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = record(first, last, sl, s, seg + 1 < ncp ? h->state : nullptr);
        }
    }
    if (e == cudaSuccess) e = gather3(h, h->ybin, Apb, Amb, A0b, s);
    if (e == cudaSuccess && pipelined) {
        e = cudaEventRecord(h->fwdDone, s);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventRecord(h->slotFree[i], s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->adjStream, h->fwdDone, 0);
    }
    // backward, one segment at a time; segment seg-1 is recomputed from its
    // checkpoint (on the side stream when pipelined) while segment seg steps the
    // cotangent back.  The cotangent alternates between two buffers.
    double* ybCur = h->ybin;
    double* ybNext = h->ybAlt;
    for (int seg = ncp - 1; seg >= 0 && e == cudaSuccess; --seg) {
        const int first = seg * K, last = std::min(n, first + K);
        const int sl = slotOf(seg);
        if (pipelined) {
            if (seg >= 1) {
                const int ps = slotOf(seg - 1), pf = (seg - 1) * K, pl = std::min(n, pf + K);
                if (seg - 1 == directSeg) {
                    e = cudaEventRecord(h->slotReady[ps], s);  // recorded by the forward pass on this stream
                } else {
                    e = cudaStreamWaitEvent(h->adjStream, h->slotFree[ps], 0);
                    if (e == cudaSuccess)
                        e = cudaMemcpyAsync(h->segment[4 * K * ps], h->checkpoints[seg - 1], stateBytes,
                                            cudaMemcpyDeviceToDevice, h->adjStream);
                    if (e == cudaSuccess) e = record(pf, pl, ps, h->adjStream, nullptr);
                    if (e == cudaSuccess) e = cudaEventRecord(h->slotReady[ps], h->adjStream);
                }
            }
            if (e == cudaSuccess && seg + 1 < ncp) e = cudaStreamWaitEvent(s, h->slotReady[sl], 0);
        } else if (seg + 1 < ncp) {
            e = cudaMemcpyAsync(h->segment[0], h->checkpoints[seg], stateBytes, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = record(first, last, 0, s, nullptr);
        }
        for (int i = last - 1; i >= first && e == cudaSuccess; --i) {
            double** q = h->segment.data() + 4 * K * sl + 4 * (i - first);
            void* const* ys = keepY ? h->ystore.data() + 4 * K * sl + 4 * (i - first) : nullptr;
            e = rk4_backward(h, q[0], q[1], q[2], q[3], times[i], t0, dt, ybCur, s, ys, ybNext);
            std::swap(ybCur, ybNext);
        }
        if (e == cudaSuccess && pipelined) e = cudaEventRecord(h->slotFree[sl], s);
    }
    if (e == cudaSuccess) e = scatter3(h, ybCur, Apb, Amb, A0b, s);
    return finish(h, e, "RK4 adjoint");
}


// Flux on the static scratch array: no cudaMalloc, cudaFree or allocating
// library call.  See include/wvgpu.h for who needs it and its limits.
int wv_nonlinear_flux_device_noalloc(wv_handle* h, double t, double t0, const double* Ap, const double* Am,
                                     const double* A0, double* Fp, double* Fm, double* F0, void* stream) {
    if (!h) return WV_INVALID_POINTER;
    int rc = check_times(h, t, t0); if (rc) return rc;
    rc = check_state_flux(h, Ap, Am, A0, Fp, Fm, F0); if (rc) return rc;
    // the static layout holds one state's scratch
    if (h->dd.members != 1)
        return fail(h, WV_UNSUPPORTED_OPERATION, "The static-scratch flux serves single-state handles only.");
    size_t offs[5];
    const size_t need = static_scratch_layout(h->plan, 2 * elem_size(h->precision), offs);
    if (need > kStaticScratchBytes)
        return fail(h, WV_SIZE_OVERFLOW, "This configuration needs " + std::to_string(need) +
                                             " bytes of flux scratch; the static scratch array holds " +
                                             std::to_string(kStaticScratchBytes) + " bytes.");
    Guard g(h->busy);
    if (!g.entered) return fail(h, WV_REENTRANT_EXECUTION, "Kernel operations are not reentrant.");
    cudaError_t e = cudaSetDevice(h->device);
    void* base = nullptr;
    if (e == cudaSuccess) e = static_scratch_address(h->device, &base);
    if (e != cudaSuccess) return cuda_fail(h, e, "static scratch set-up");
    auto s = static_cast<cudaStream_t>(stream);
    unsigned char* sb = static_cast<unsigned char*>(base);
    const FluxScratch sc{sb + offs[0], sb + offs[1], sb + offs[2], sb + offs[3],
                         reinterpret_cast<unsigned long long*>(sb + offs[4])};
    // the same launch sequence (and kernel choice) as wv_nonlinear_flux_device, without damping
    e = h->precision == WV_PRECISION_FP64
            ? launch_flux<double>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, s, nullptr, nullptr, nullptr, &sc)
        : h->precision == WV_PRECISION_MIXED
            ? launch_flux<float>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, s, nullptr, nullptr, nullptr, &sc)
            : launch_flux<dev::ff>(h, t, t0, Ap, Am, A0, Fp, Fm, F0, false, s, nullptr, nullptr, nullptr, &sc);
    h->metrics.nonlinear_flux_calls++;
    return finish(h, e, "nonlinear flux (static scratch)");
}

}  // extern "C"

// ---- ensembles ----------------------------------------------------------------------
// Groups of states on uneven grids.  Each group is one member-batched handle
// (all its members' planes and columns in one launch per stage); every group
// runs on its own stream forked from the ensemble's capture stream, and the
// whole n-step integration of all groups is captured once into a CUDA graph and
// replayed with one cudaGraphLaunch.  No counterpart in the reference, which
// steps one state per kernel object.

struct wv_ensemble {
    std::vector<wv_handle*> groups;
    std::vector<int> members;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaStream_t capture = nullptr;
    cudaGraphExec_t exec = nullptr;
    // what the instantiated graph was captured for
    std::vector<double*> keyStates;
    std::vector<double> keyDt, keyT;
    double keyT0 = 0.0;
    int keySteps = -1;
    std::vector<wv_ensemble_tuning> tuning;
    wv_ensemble_metrics metrics{};
    std::atomic<bool> busy{false};
    int device = 0;
    std::string message;
};

namespace {

int efail(wv_ensemble* e, int code, const std::string& m) {
    if (e) e->message = m;
    return code;
}

// Device time (ms) of `reps` fluxes of one group on its own buffers.
float time_group_flux(wv_handle* h, int reps, cudaStream_t s, cudaError_t& err) {
    const size_t M2 = 2 * h->plan.M;
    cudaEvent_t a = nullptr, b = nullptr;
    err = cudaEventCreate(&a);
    if (err == cudaSuccess) err = cudaEventCreate(&b);
    float ms = 0.0f;
    if (err == cudaSuccess) err = flux_any(h, 0.0, 0.0, h->state, h->state + M2, h->state + 2 * M2, h->kbuf, h->kbuf + M2,
                                           h->kbuf + 2 * M2, false, s);
    if (err == cudaSuccess) err = cudaEventRecord(a, s);
    for (int r = 0; r < reps && err == cudaSuccess; ++r)
        err = flux_any(h, 0.0, 0.0, h->state, h->state + M2, h->state + 2 * M2, h->kbuf, h->kbuf + M2, h->kbuf + 2 * M2,
                       false, s);
    if (err == cudaSuccess) err = cudaEventRecord(b, s);
    if (err == cudaSuccess) err = cudaEventSynchronize(b);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    return ms / static_cast<float>(reps > 0 ? reps : 1);
}

// Per group, the fastest of the FFT variants that exist for its grid: the
// register-resident warp FFT or the shared-memory Stockham kernel, per axis
// (whole-flux times); then, for mixed groups, the fastest kernel of each
// vertical transform direction (dense contraction, FFTs, tensor cores: what the
// grid has), from the stage times of the flux.  FP32X2 and FP64 groups keep the
// handle's vertical kernels, so that members stay bit-identical to single
// handles of those precisions.
cudaError_t autotune_group(wv_handle* h, cudaStream_t s, wv_ensemble_tuning& out) {
    cudaError_t e = cudaMemsetAsync(h->state, 0, 6 * h->plan.M * h->dd.members * sizeof(double), s);
    Plan& p = h->plan;
    // FP32X2 and FP64 groups keep the handle's FFT variants (bit-identical members)
    const bool fp32 = h->precision == WV_PRECISION_MIXED;
    const bool warpY = fp32 && warp_ry<float>(p) != 0, warpX = fp32 && warp_rx<float>(p) != 0;
    float best = -1.0f;
    bool bestY = false, bestX = false;
    out.candidates = 0;
    for (int vy = 0; vy < (warpY ? 2 : 1) && e == cudaSuccess; ++vy) {
        for (int vx = 0; vx < (warpX ? 2 : 1) && e == cudaSuccess; ++vx) {
            p.stockhamY = vy == 1;
            p.stockhamX = vx == 1;
            const float ms = time_group_flux(h, 3, s, e);
            if (e == cudaSuccess && out.candidates < WV_ENSEMBLE_MAX_CANDIDATES) out.candidate_ms[out.candidates] = ms;
            out.candidates++;
            if (e == cudaSuccess && (best < 0.0f || ms < best)) { best = ms; bestY = p.stockhamY; bestX = p.stockhamX; }
        }
    }
    p.stockhamY = bestY;
    p.stockhamX = bestX;
    for (int k = 0; k < 3; ++k) out.vertical_inverse_ms[k] = out.vertical_forward_ms[k] = -1.0f;
    if (h->precision == WV_PRECISION_MIXED && e == cudaSuccess) {
        const int kinds[3] = {WV_VERTICAL_CUDA_CORES, WV_VERTICAL_FFT, WV_VERTICAL_TENSOR_CORES};
        const bool has[3] = {true, p.fz.N > 0, h->tcAvailable};
        const bool hasFwd[3] = {true, p.fz.N > 0, h->tcFwdAvailable};
        const size_t M2 = 2 * p.M;
        const bool inst = h->instrument;
        const wv_stage_times keep = h->stages;
        if (wv_set_stage_instrumentation(h, 1) != WV_SUCCESS) e = cudaErrorUnknown;
        for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
            if (!has[k]) continue;
            h->vinvKind = kinds[k];
            h->vfwdKind = hasFwd[k] ? kinds[k] : WV_VERTICAL_CUDA_CORES;
            e = flux_any(h, 0.0, 0.0, h->state, h->state + M2, h->state + 2 * M2, h->kbuf, h->kbuf + M2, h->kbuf + 2 * M2,
                         false, s);  // warm-up
            h->stages = wv_stage_times{};
            for (int r = 0; r < 3 && e == cudaSuccess; ++r)
                e = flux_any(h, 0.0, 0.0, h->state, h->state + M2, h->state + 2 * M2, h->kbuf, h->kbuf + M2, h->kbuf + 2 * M2,
                             false, s);
            if (e != cudaSuccess) break;
            const double n = static_cast<double>(h->stages.fluxes > 0 ? h->stages.fluxes : 1);
            out.vertical_inverse_ms[kinds[k]] = static_cast<float>(h->stages.vertical_inverse_ms / n);
            if (hasFwd[k]) out.vertical_forward_ms[kinds[k]] = static_cast<float>(h->stages.vertical_forward_ms / n);
        }
        h->instrument = inst;
        h->stages = keep;
        // fastest of each direction (index WV_VERTICAL_*; the dense kernel always exists)
        int bi = WV_VERTICAL_CUDA_CORES, bf = WV_VERTICAL_CUDA_CORES;
        for (int k = 0; k < 3; ++k) {
            if (out.vertical_inverse_ms[k] >= 0.0f && out.vertical_inverse_ms[k] < out.vertical_inverse_ms[bi]) bi = k;
            if (out.vertical_forward_ms[k] >= 0.0f && out.vertical_forward_ms[k] < out.vertical_forward_ms[bf]) bf = k;
        }
        h->vinvKind = bi;
        h->vfwdKind = bf;
        if (e == cudaSuccess) best = time_group_flux(h, 3, s, e);
    }
    out.stockham_y = bestY ? 1 : 0;
    out.stockham_x = bestX ? 1 : 0;
    out.vertical = h->vinvKind;
    out.vertical_forward = h->vfwdKind;
    out.warp_y_available = warpY ? 1 : 0;
    out.warp_x_available = warpX ? 1 : 0;
    out.tensor_vertical_available = h->tcAvailable ? 1 : 0;
    out.flux_ms = best;
    return e;
}

}  // namespace

extern "C" {

void wv_ensemble_destroy(wv_ensemble* e) {
    if (!e) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(e->device);
    if (e->capture) cudaStreamSynchronize(e->capture);
    for (cudaStream_t st : e->side) if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
    if (e->exec) cudaGraphExecDestroy(e->exec);
    for (cudaEvent_t ev : e->join) if (ev) cudaEventDestroy(ev);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->capture) cudaStreamDestroy(e->capture);
    for (wv_handle* h : e->groups) wv_destroy(h);
    cudaSetDevice(prev);
    delete e;
}

int wv_ensemble_create(const wv_config* group_configs, const int* members, int n_groups, int precision, int autotune,
                       wv_ensemble** out) {
    if (!out) return WV_INVALID_POINTER;
    *out = nullptr;
    if (!group_configs || !members) return WV_INVALID_POINTER;
    if (n_groups < 1 || n_groups > WV_ENSEMBLE_MAX_GROUPS) return WV_INVALID_CONFIGURATION;
    for (int g = 0; g < n_groups; ++g) if (members[g] < 1) return WV_INVALID_CONFIGURATION;
    wv_ensemble* e = new (std::nothrow) wv_ensemble();
    if (!e) return WV_ALLOCATION_FAILURE;
    cudaGetDevice(&e->device);
    for (int g = 0; g < n_groups; ++g) {
        wv_handle* h = nullptr;
        const int rc = create_handle(&group_configs[g], precision, members[g], &h);
        if (rc) { wv_ensemble_destroy(e); return rc; }
        e->groups.push_back(h);
        e->members.push_back(members[g]);
    }
    cudaError_t err = cudaStreamCreateWithFlags(&e->capture, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    for (int g = 0; g < n_groups && err == cudaSuccess; ++g) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        e->side.push_back(st);
        e->join.push_back(ev);
    }
    e->tuning.assign(n_groups, wv_ensemble_tuning{});
    for (int g = 0; g < n_groups && err == cudaSuccess; ++g) {
        wv_handle* h = e->groups[g];
        if (autotune) {
            err = autotune_group(h, e->capture, e->tuning[g]);
        } else {
            wv_ensemble_tuning& t = e->tuning[g];
            t.stockham_y = h->plan.stockhamY ? 1 : 0;
            t.stockham_x = h->plan.stockhamX ? 1 : 0;
            t.warp_y_available = h->precision == WV_PRECISION_MIXED && warp_ry<float>(h->plan) != 0;
            t.warp_x_available = h->precision == WV_PRECISION_MIXED && warp_rx<float>(h->plan) != 0;
            t.tensor_vertical_available = h->tcAvailable ? 1 : 0;
            t.vertical = h->vinvKind;
            t.vertical_forward = h->vfwdKind;
            for (int k = 0; k < 3; ++k) t.vertical_inverse_ms[k] = t.vertical_forward_ms[k] = -1.0f;
            t.flux_ms = -1.0f;
        }
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->capture);
    if (err != cudaSuccess) {
        const int code = err == cudaErrorMemoryAllocation ? WV_ALLOCATION_FAILURE : WV_FFT_PLAN_FAILURE;
        wv_ensemble_destroy(e);
        return code;
    }
    size_t bytes = 0;
    for (wv_handle* h : e->groups) bytes += h->deviceBytes;
    e->metrics.device_bytes = bytes;
    *out = e;
    return WV_SUCCESS;
}

const char* wv_ensemble_last_message(const wv_ensemble* e) { return e ? e->message.c_str() : "null ensemble"; }

int wv_ensemble_get_sizes(const wv_ensemble* e, int group, wv_sizes* sizes) {
    if (!e || !sizes) return WV_INVALID_POINTER;
    if (group < 0 || group >= static_cast<int>(e->groups.size())) return WV_INVALID_CONFIGURATION;
    return wv_get_sizes(e->groups[group], sizes);
}

int wv_ensemble_get_tuning(const wv_ensemble* e, int group, wv_ensemble_tuning* tuning) {
    if (!e || !tuning) return WV_INVALID_POINTER;
    if (group < 0 || group >= static_cast<int>(e->groups.size())) return WV_INVALID_CONFIGURATION;
    *tuning = e->tuning[group];
    return WV_SUCCESS;
}

int wv_ensemble_set_vertical_kernel(wv_ensemble* e, int kind) {
    if (!e) return WV_INVALID_POINTER;
    if (kind != WV_VERTICAL_CUDA_CORES && kind != WV_VERTICAL_TENSOR_CORES && kind != WV_VERTICAL_FFT)
        return efail(e, WV_INVALID_CONFIGURATION, "Unknown vertical-transform kernel.");
    for (wv_handle* h : e->groups)
        if (kind == WV_VERTICAL_FFT && h->plan.fz.N == 0)
            return efail(e, WV_UNSUPPORTED_OPERATION, "The FFT vertical transform needs groups with 3 <= Nz <= 513.");
    for (wv_handle* h : e->groups)
        if (kind == WV_VERTICAL_TENSOR_CORES && !h->tcAvailable)
            return efail(e, WV_UNSUPPORTED_OPERATION,
                         "The tensor-core vertical transform needs mixed-precision (Nz <= 255) or FP32X2 (Nj <= 96) groups.");
    for (size_t g = 0; g < e->groups.size(); ++g) {
        wv_handle* h = e->groups[g];
        h->vinvKind = kind;
        h->vfwdKind = kind == WV_VERTICAL_TENSOR_CORES && !h->tcFwdAvailable ? WV_VERTICAL_CUDA_CORES : kind;
        e->tuning[g].vertical = h->vinvKind;
        e->tuning[g].vertical_forward = h->vfwdKind;
    }
    e->keySteps = -1;  // captured kernels changed: capture anew
    return WV_SUCCESS;
}

int wv_ensemble_get_metrics(const wv_ensemble* e, wv_ensemble_metrics* m) {
    if (!e || !m) return WV_INVALID_POINTER;
    *m = e->metrics;
    return WV_SUCCESS;
}

int wv_ensemble_rk4_device(wv_ensemble* e, double* const* states, double* t, double t0, const double* dt, int n,
                           void* stream) {
    if (!e) return WV_INVALID_POINTER;
    if (!states || !t || !dt) return efail(e, WV_INVALID_POINTER, "Ensemble RK4 received a null pointer.");
    const int G = static_cast<int>(e->groups.size());
    if (!std::isfinite(t0)) return efail(e, WV_INVALID_CONFIGURATION, "Times must be finite.");
    for (int g = 0; g < G; ++g)
        if (!std::isfinite(t[g])) return efail(e, WV_INVALID_CONFIGURATION, "Times must be finite.");
    if (n < 0) return efail(e, WV_INVALID_CONFIGURATION, "RK4 step count must be nonnegative.");
    for (int g = 0; g < G; ++g) {
        if (!states[g]) return efail(e, WV_INVALID_POINTER, "Ensemble RK4 received a null group state.");
        if (!(dt[g] > 0.0) || !std::isfinite(dt[g]))
            return efail(e, WV_INVALID_CONFIGURATION, "RK4 step sizes must be finite and positive.");
        if (reinterpret_cast<uintptr_t>(states[g]) % 16)
            return efail(e, WV_INVALID_POINTER, "Group states must be 16-byte aligned complex arrays.");
        for (int q = 0; q < g; ++q) {
            const size_t bg = 6 * e->groups[g]->plan.M * e->members[g] * sizeof(double);
            const size_t bq = 6 * e->groups[q]->plan.M * e->members[q] * sizeof(double);
            if (overlaps(states[g], bg, states[q], bq)) return efail(e, WV_OVERLAPPING_ARRAYS, "Group states overlap.");
        }
    }
    if (n == 0) return WV_SUCCESS;
    Guard guard(e->busy);
    if (!guard.entered) return efail(e, WV_REENTRANT_EXECUTION, "Ensemble stepping is not reentrant.");
    cudaSetDevice(e->device);
    // step times exactly as WVFixedStepRK4 advances them, per group
    std::vector<double> tEnd(t, t + G);
    const bool same = e->exec && e->keySteps == n && e->keyT0 == t0 && static_cast<int>(e->keyDt.size()) == G &&
                      std::equal(e->keyDt.begin(), e->keyDt.end(), dt) && std::equal(e->keyT.begin(), e->keyT.end(), t) &&
                      std::equal(e->keyStates.begin(), e->keyStates.end(), states);
    cudaError_t err = cudaSuccess;
    if (!same) {
        cudaGraph_t graph = nullptr;
        err = cudaStreamBeginCapture(e->capture, cudaStreamCaptureModeThreadLocal);
        if (err == cudaSuccess) err = cudaEventRecord(e->fork, e->capture);
        for (int g = 0; g < G && err == cudaSuccess; ++g) {
            wv_handle* h = e->groups[g];
            cudaStream_t s = e->side[g];
            const size_t bytes = 6 * h->plan.M * e->members[g] * sizeof(double);
            err = cudaStreamWaitEvent(s, e->fork, 0);
            if (err == cudaSuccess) err = cudaMemcpyAsync(h->state, states[g], bytes, cudaMemcpyDeviceToDevice, s);
            double tt = t[g];
            for (int i = 0; i < n && err == cudaSuccess; ++i) {
                err = rk4_step(h, tt, t0, dt[g], s);
                tt = tt + dt[g];
            }
            if (err == cudaSuccess) err = cudaMemcpyAsync(states[g], h->state, bytes, cudaMemcpyDeviceToDevice, s);
            if (err == cudaSuccess) err = cudaEventRecord(e->join[g], s);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(e->capture, e->join[g], 0);
        }
        const cudaError_t endErr = cudaStreamEndCapture(e->capture, &graph);
        if (err == cudaSuccess) err = endErr;
        if (err == cudaSuccess) {
            // same topology (same groups and step count): update the parameters in place
            bool updated = false;
            if (e->exec && e->keySteps == n) {
                cudaGraphExecUpdateResultInfo info{};
                updated = cudaGraphExecUpdate(e->exec, graph, &info) == cudaSuccess;
                if (!updated) cudaGetLastError();
            }
            if (!updated) {
                if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
                err = cudaGraphInstantiate(&e->exec, graph, 0);
                e->metrics.graph_instantiations++;
            } else {
                e->metrics.graph_updates++;
            }
            e->metrics.graph_captures++;
        }
        if (graph) cudaGraphDestroy(graph);
        if (err != cudaSuccess) {
            if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
            e->keySteps = -1;
            return efail(e, WV_FFT_EXECUTION_FAILURE, std::string("ensemble graph capture: ") + cudaGetErrorString(err));
        }
        e->keyStates.assign(states, states + G);
        e->keyDt.assign(dt, dt + G);
        e->keyT.assign(t, t + G);
        e->keyT0 = t0;
        e->keySteps = n;
    }
    err = cudaGraphLaunch(e->exec, static_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return efail(e, WV_FFT_EXECUTION_FAILURE, std::string("ensemble graph launch: ") + cudaGetErrorString(err));
    e->metrics.graph_launches++;
    unsigned long long launches = 0;
    for (int g = 0; g < G; ++g) {
        launches += static_cast<unsigned long long>(n) * 25;
        e->metrics.member_steps += static_cast<unsigned long long>(n) * e->members[g];
    }
    e->metrics.kernel_launches += launches;
    for (int g = 0; g < G; ++g) {
        double tt = t[g];
        for (int i = 0; i < n; ++i) tt = tt + dt[g];
        t[g] = tt;
    }
    return WV_SUCCESS;
}

}  // extern "C"

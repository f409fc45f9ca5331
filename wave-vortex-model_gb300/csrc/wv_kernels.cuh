// CUDA kernels of the constant-stratification spectral step (sm_103a).
//
// Pipeline of one nonlinear flux (nonlinearFluxImpl, kernel.cpp:1173-1244),
// restructured for the GPU:
//   vinv   : per retained (k,l) column: phase, evolved coefficients, field
//            spectra (coefficientValueForField), then the vertical inverse
//            DCT-I/DST-I as a folded dense contraction -> zspec[ch][z][pos]
//   yinv   : per (z, kx): inverse FFT along y of each channel (and of i*l*q)
//            -> yspec[z][ch][y][kx]
//   xflux  : per (z, y) row: c2r along x of U,V,W and every derivative,
//            quadratic products S_q = -(u q_x + v q_y + w q_z), max |u_h|,
//            r2c of S_q along x -> pspec[z][q][y][kx]
//   yfwd   : per (z, kx): forward FFT along y, gathered to active rows -> fspec
//   vfwd   : per column: forward DCT-I/DST-I contraction, projection onto
//            Ap/Am/A0 (projectFluxTargetMode, kernel.cpp:396-431), phase,
//            adaptive damping, written as Fp/Fm/F0.
// T is the working type of the xy stage and the vertical contractions
// (double for FP64 handles, float for MIXED, the paired-FP32 ff for FP32X2);
// phases, projections and accumulations are always double.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "wv_ff.cuh"

namespace wvgpu {
namespace dev {

template <typename T> struct cxt;
template <> struct cxt<double> { using type = double2; };
template <> struct cxt<float> { using type = float2; };
template <> struct cxt<ff> { using type = ff2; };
template <typename T> using cx = typename cxt<T>::type;
// Minimum resident CTAs of the vertical forward kernel: paired FP32 trades a
// few registers for a third CTA per SM (its FP32-pipe chains need the warps).
template <typename T> struct VertOcc { static constexpr int value = 1; };
template <> struct VertOcc<ff> { static constexpr int value = 3; };

template <typename T> __device__ __forceinline__ cx<T> mk(T a, T b) { cx<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) { return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename T> __device__ __forceinline__ cx<T> cconj(cx<T> a) { return mk<T>(a.x, -a.y); }
template <typename T> __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
#ifdef __CUDACC__
// FP32 complex sums on the paired FP32 instructions of sm_100+ (FADD2: both
// components in one instruction, each rounded as its scalar add)
template <> __device__ __forceinline__ cx<float> cadd<float>(cx<float> a, cx<float> b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ cx<float> csub<float>(cx<float> a, cx<float> b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
#endif
// multiply by +i (INV) or -i (forward) : used by radix-4 butterflies
template <bool INV, typename T> __device__ __forceinline__ cx<T> mul_mi(cx<T> a) { return INV ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x); }

// Exact complex arithmetic of the reference (no contraction), double only.
struct zd { double re, im; };
__device__ __forceinline__ zd zmul(zd a, zd b) {
    return {__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)), __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re))};
}
__device__ __forceinline__ zd zadd(zd a, zd b) { return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }
__device__ __forceinline__ zd zsub(zd a, zd b) { return {__dsub_rn(a.re, b.re), __dsub_rn(a.im, b.im)}; }
__device__ __forceinline__ zd zscale(zd a, double s) { return {__dmul_rn(a.re, s), __dmul_rn(a.im, s)}; }
__device__ __forceinline__ zd zconj(zd a) { return {a.re, -a.im}; }
__device__ __forceinline__ zd zload(const double* p) { const double2 v = *reinterpret_cast<const double2*>(p); return {v.x, v.y}; }
__device__ __forceinline__ void zstore(double* p, zd v) { *reinterpret_cast<double2*>(p) = make_double2(v.re, v.im); }

constexpr int kMaxStages = 24;

struct FFTDev {
    int N;
    int nstages;
    int radix[kMaxStages];
};

// ---------------------------------------------------------------------------
// Shared-memory Stockham FFT over `lines` lines of length N (leading dim ld).
// Forward uses exp(-2 pi i k/N), inverse the conjugate; both unnormalized.

template <typename T, bool INV>
__device__ __forceinline__ cx<T> twid(const cx<T>* tw, int idx) {
    cx<T> w = tw[idx];
    return INV ? cconj<T>(w) : w;
}

// Work item `it` of a stage -> (line, j = index within the line's nb butterflies,
// k = j mod Ns, j / Ns).  Power-of-two lengths (every radix 2 or 4, so nb and Ns
// are powers of two) use shifts and masks: integer division costs tens of
// instructions, which the FP32-issue-bound paired-FP32 lines pay per butterfly.
struct StageIdx {
    int line, j, k, jq;
};
__device__ __forceinline__ StageIdx stage_idx(int it, int nb, int Ns, bool p2, int nbShift, int nsShift) {
    StageIdx r;
    if (p2) {
        r.line = it >> nbShift;
        r.j = it & (nb - 1);
        r.k = r.j & (Ns - 1);
        r.jq = r.j >> nsShift;
    } else {
        r.line = it / nb;
        r.j = it - r.line * nb;
        r.k = r.j % Ns;
        r.jq = r.j / Ns;
    }
    return r;
}

template <typename T, bool INV>
__device__ void fft_stage(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst, int N, int R, int Ns, int lines, int ld,
                          const cx<T>* __restrict__ tw) {
    const int nb = N / R;
    const int tstride = N / (Ns * R);
    const bool p2 = (N & (N - 1)) == 0;
    const int nbShift = __ffs(nb) - 1, nsShift = __ffs(Ns) - 1;
    if (R == 4) {
        for (int it = threadIdx.x; it < lines * nb; it += blockDim.x) {
            const StageIdx ix = stage_idx(it, nb, Ns, p2, nbShift, nsShift);
            const int line = ix.line, j = ix.j;
            const cx<T>* in = src + line * ld;
            cx<T>* out = dst + line * ld;
            const int k = ix.k;
            const int ts = k * tstride;
            cx<T> v0 = in[j], v1 = in[j + nb], v2 = in[j + 2 * nb], v3 = in[j + 3 * nb];
            if (ts) {
                v1 = cmul<T>(v1, twid<T, INV>(tw, ts));
                v2 = cmul<T>(v2, twid<T, INV>(tw, 2 * ts));
                v3 = cmul<T>(v3, twid<T, INV>(tw, 3 * ts));
            }
            const cx<T> a = cadd<T>(v0, v2), b = csub<T>(v0, v2), c = cadd<T>(v1, v3), d = mul_mi<INV, T>(csub<T>(v1, v3));
            const int o = ix.jq * Ns * 4 + k;
            out[o] = cadd<T>(a, c);
            out[o + Ns] = cadd<T>(b, d);
            out[o + 2 * Ns] = csub<T>(a, c);
            out[o + 3 * Ns] = csub<T>(b, d);
        }
    } else if (R == 2) {
        for (int it = threadIdx.x; it < lines * nb; it += blockDim.x) {
            const StageIdx ix = stage_idx(it, nb, Ns, p2, nbShift, nsShift);
            const int line = ix.line, j = ix.j;
            const cx<T>* in = src + line * ld;
            cx<T>* out = dst + line * ld;
            const int k = ix.k;
            const int ts = k * tstride;
            cx<T> v0 = in[j], v1 = in[j + nb];
            if (ts) v1 = cmul<T>(v1, twid<T, INV>(tw, ts));
            const int o = ix.jq * Ns * 2 + k;
            out[o] = cadd<T>(v0, v1);
            out[o + Ns] = csub<T>(v0, v1);
        }
    } else if (R == 3) {
        const T s3 = INV ? T(0.86602540378443864676) : T(-0.86602540378443864676);
        for (int it = threadIdx.x; it < lines * nb; it += blockDim.x) {
            const int line = it / nb, j = it - line * nb;
            const cx<T>* in = src + line * ld;
            cx<T>* out = dst + line * ld;
            const int k = j % Ns;
            const int ts = k * tstride;
            cx<T> v0 = in[j], v1 = in[j + nb], v2 = in[j + 2 * nb];
            if (ts) {
                v1 = cmul<T>(v1, twid<T, INV>(tw, ts));
                v2 = cmul<T>(v2, twid<T, INV>(tw, 2 * ts));
            }
            const cx<T> t1 = cadd<T>(v1, v2);
            const cx<T> t2 = mk<T>(v0.x - T(0.5) * t1.x, v0.y - T(0.5) * t1.y);
            const cx<T> dlt = csub<T>(v1, v2);
            const cx<T> t3 = mk<T>(-s3 * dlt.y, s3 * dlt.x);  // i * s3 * (v1 - v2)
            const int o = (j / Ns) * Ns * 3 + k;
            out[o] = cadd<T>(v0, t1);
            out[o + Ns] = cadd<T>(t2, t3);
            out[o + 2 * Ns] = csub<T>(t2, t3);
        }
    } else {
        // Generic radix: one output per work item, O(R) dot product.
        for (int it = threadIdx.x; it < lines * N; it += blockDim.x) {
            const int line = it / N, rem = it - line * N;
            const int j = rem % nb, r = rem / nb;
            const cx<T>* in = src + line * ld;
            cx<T>* out = dst + line * ld;
            const int k = j % Ns;
            const int step = (k * tstride + r * nb) % N;
            cx<T> acc = mk<T>(T(0), T(0));
            int e = 0;
            for (int m = 0; m < R; ++m) {
                acc = cadd<T>(acc, cmul<T>(in[j + m * nb], twid<T, INV>(tw, e)));
                e += step;
                if (e >= N) e -= N;
            }
            out[(j / Ns) * Ns * R + k + r * Ns] = acc;
        }
    }
}

// Runs all stages; returns the buffer holding the result (a or b).
template <typename T, bool INV>
__device__ cx<T>* fft_lines(cx<T>* a, cx<T>* b, const FFTDev& f, int lines, int ld, const cx<T>* tw) {
    int Ns = 1;
    for (int s = 0; s < f.nstages; ++s) {
        fft_stage<T, INV>(a, b, f.N, f.radix[s], Ns, lines, ld, tw);
        __syncthreads();
        Ns *= f.radix[s];
        cx<T>* t = a; a = b; b = t;
    }
    return a;
}

// ---------------------------------------------------------------------------
// Parameters shared by the kernels of one handle.

struct DescDev {
    int Nx, Ny, Nz, Nj, Nkl, NxHalf, M;
    int positions, kxColumns, zHalf;
    int nt;          // number of flux targets
    int tq[4];       // target ids (0=u,1=v,2=w,3=eta)
    int hydrostatic;
    // Ensemble batching: `members` states of this grid side by side, member m's
    // coefficients at m*memberStride doubles; column buffers [ch][m*Nz+z][pos]
    // and plane buffers [m*Nz+z][...], so zTotal = members*Nz planes.  A single
    // state is members = 1.
    int members, zTotal;
    long long memberStride;
    // descriptor arrays [M] (j fastest)
    const double* omega;
    const double* UAp;   // complex interleaved
    const double* VAp;
    const double* WAp;
    const double* NAp;
    const double* UA0;
    const double* VA0;
    const double* NA0;
    const double* A0FromVorticity;
    const double* A0FromBuoyancy;
    const double* ApmN;
    const double* ApmDScaled;
    const double* ApmD;  // complex (hydrostatic projection)
    const double* damping;  // [M] adaptive damping operator (or null)
    // FP32 copies of the field factors (MIXED handles only; complex interleaved)
    const float* fUAp;
    const float* fVAp;
    const float* fWAp;
    const float* fNAp;
    const float* fUA0;
    const float* fVA0;
    const float* fNA0;
    // per WV mode [Nkl]
    const double* k;
    const double* l;
    const double* Kh;
    const double* cosAlpha;
    const double* sinAlpha;
    // per j [Nj]
    const double* inertialScale;
    const double* apmWPrefactor;
    // plan
    const int* posKy;       // [positions]
    const int* colStart;    // [kxColumns+1]
    const int* ymap;        // [kxColumns][Ny] position of (kx, ky) or -1
    const int* modeWV;      // [Nkl] in position order
    const int* modePos;
    const int* modeCompPos;
    const unsigned char* modeFlags;
    const double* rowK;     // [kxColumns]
    const double* rowL;     // [Ny]
    const void* tRowK;      // rowK, rowL in the working type of the xy stage
    const void* tRowL;
    // MIXED handles: flux projection coefficients per (mode, j), 12 floats each:
    // Cu, Cv, Cw (complex), Du, Dv (imaginary parts), Dn, Npm, B; see k_vfwd.
    const float* fProj;
    const void* Ccos;       // T[zHalf][Nj]
    const void* Csin;
    const void* CcosM;
    const void* CsinM;
    const void* Fcos;       // T[Nj][zHalf]
    const void* Fsin;
    // transposed copies for the adjoint kernels (contiguous along their inner loop)
    const void* CcosT;      // T[Nj][zHalf]
    const void* CsinT;
    const void* CcosMT;
    const void* CsinMT;
    const void* FcosT;      // T[zHalf][Nj]
    const void* FsinT;
    const void* twx;        // cx<T>[xLen]: twiddles of the x line FFT (length Nx/2 for even Nx, else Nx)
    const void* twxN;       // cx<T>[Nx]: exp(-2 pi i k/Nx) for the real-FFT split/merge
    const void* twy;        // cx<T>[Ny]
    // MIXED handles with the tensor-core vertical transform: the four folded
    // inverse matrices split into three BF16 pieces each, in the canonical
    // no-swizzle K-major layout [matrix][piece][N rows][K]; N = Zh rounded up to
    // 16, K = KE (even j) + odd j, each rounded up to 16.
    const unsigned short* tcB;
    int tcN, tcKE, tcK;
    // ... and the forward matrices Fcos, Fsin split by output parity:
    // [family cos|sin][parity even|odd][piece][NF rows j/2][KF = Zh rounded up to 16]
    const unsigned short* tcFB;
    int tcFN, tcFK;
    // FP32X2 handles with the tensor-core vertical inverse: the matrices Ccos,
    // Csin, Ccos, -Csin (the last two are the z-derivative matrices with m_j moved
    // into the A operand) as six signed 8-bit digit slices per row (BF16, slice t
    // scaled by 2^(-7-8t), row n scaled by 2^-tcxF[m][n]), blocks [matrix][j parity]
    // [pass][slice][tcxN rows][tcxKH], output rows n = pass tcxN + row
    const unsigned short* tcxB;
    const int* tcxF;        // [4][tcxPasses tcxN] row exponents
    const void* tcxM;       // ff[Nj]: m_j
    int tcxN, tcxKH, tcxPasses;
    unsigned* status;       // device status word (bit 0: a bounded wait ran out)
    unsigned injectWaitPolls;  // test hook (0: off): k_vinv_tc's first operand wait gets no copy and this poll limit
    int c2rUseK;            // k_xc2r_fields(_w): bit c set -> channel c is multiplied by i k (x derivative)
    // field-family scales (transformToSpatialDomainWith{F,G}AllDerivatives)
    const double* fWaveScale;   // [M]
    const double* gWaveScale;   // [Nj]
    const double* Fg;           // [Nj]
    const double* Gg;           // [Nj]
    int xEven;              // Nx even: real rows go through half-length complex FFTs
    int xLen;               // Nx/2 (even) or Nx (odd)
    FFTDev fx, fy;          // fx factors xLen
    FFTDev fz;              // 2 (Nz - 1): vertical transforms as FFTs (N = 0: not available)
    const void* twz;        // cx<T>[2 (Nz - 1)]
    const void* tMz;        // T[Nj]: m_j in the working type
};

// Row wavenumbers in the working type T of the xy stage.
template <typename T>
__device__ __forceinline__ const T* row_k(const DescDev& d) { return static_cast<const T*>(d.tRowK); }
template <typename T>
__device__ __forceinline__ const T* row_l(const DescDev& d) { return static_cast<const T*>(d.tRowL); }


// ---------------------------------------------------------------------------
// vinv: evolved field spectra + vertical inverse contraction.
//   mode FIELDS: channels U, V, W, N (transformWaveVortexToUVWEta)
//   mode FLUX:   channels U, V, W, N, then d/dz of each flux target.
// Column values are in the stored frame: conjugated for kMode < 0 storage,
// imaginary part cleared on self-conjugate rows (kernel.cpp:211-291,433-438).

constexpr int kVinvModes = 8;

// Field spectra u, v, w, eta of one (mode, j) in the stored frame and working
// precision T (k_vinv's phase 1): phase (kernel.cpp:1186-1191), evolution and
// coefficient formulas (WVCoefficientFormulas.hpp:23-58), conjugated for
// kMode < 0 storage, imaginary part cleared on self-conjugate rows.
template <typename T>
__device__ __forceinline__ void vinv_field_spectra(const DescDev& d, const double* __restrict__ Ap,
                                                   const double* __restrict__ Am, const double* __restrict__ A0,
                                                   double elapsed, int mode, int j, cx<T> (&f)[4]) {
    const int Nj = d.Nj;
    const int w = d.modeWV[mode];
    const unsigned char flags = d.modeFlags[mode];
    const int idx = j + Nj * w;
    if constexpr (sizeof(T) == 4) {
        // MIXED: phase angle in FP64 reduced to [-pi, pi], then FP32 phase and field spectra.
        const double ang = d.omega[idx] * elapsed;
        const double red = ang - 6.283185307179586476925 * rint(ang * 0.15915494309189533577);
        float sf, cf;
        sincosf(float(red), &sf, &cf);
        const float2 ap0 = make_float2(float(Ap[2 * idx]), float(Ap[2 * idx + 1]));
        const float2 am0 = make_float2(float(Am[2 * idx]), float(Am[2 * idx + 1]));
        const float2 a0 = make_float2(float(A0[2 * idx]), float(A0[2 * idx + 1]));
        const float2 ap = make_float2(ap0.x * cf - ap0.y * sf, ap0.x * sf + ap0.y * cf);
        const float2 am = make_float2(am0.x * cf + am0.y * sf, am0.y * cf - am0.x * sf);
        const float2 uap = *reinterpret_cast<const float2*>(d.fUAp + 2 * idx);
        const float2 vap = *reinterpret_cast<const float2*>(d.fVAp + 2 * idx);
        const float2 wap = *reinterpret_cast<const float2*>(d.fWAp + 2 * idx);
        const float2 ua0 = *reinterpret_cast<const float2*>(d.fUA0 + 2 * idx);
        const float2 va0 = *reinterpret_cast<const float2*>(d.fVA0 + 2 * idx);
        const float nap = d.fNAp[idx], na0 = d.fNA0[idx];
        auto cm2 = [](float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto cj = [](float2 a) { return make_float2(a.x, -a.y); };
        auto ca = [](float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); };
        float2 u = ca(ca(cm2(uap, ap), cm2(cj(uap), am)), cm2(ua0, a0));
        float2 v = ca(ca(cm2(vap, ap), cm2(cj(vap), am)), cm2(va0, a0));
        float2 ww = ca(cm2(wap, ap), cm2(wap, am));
        float2 n = make_float2(ap.x * nap - am.x * nap + a0.x * na0, ap.y * nap - am.y * nap + a0.y * na0);
        if (flags & 1) { u = cj(u); v = cj(v); ww = cj(ww); n = cj(n); }
        if (flags & 2) { u.y = 0.f; v.y = 0.f; ww.y = 0.f; n.y = 0.f; }
        f[0] = mk<T>(u.x, u.y);
        f[1] = mk<T>(v.x, v.y);
        f[2] = mk<T>(ww.x, ww.y);
        f[3] = mk<T>(n.x, n.y);
        return;
    }
    if constexpr (std::is_same<T, ff>::value) {
        // FP32X2: FP64 angle, paired-FP32 phase (ff_sincos), then paired-FP32
        // evolution and field spectra with the coefficient arrays stored as
        // pairs (d.fUAp ... hold ff values)
        T sf, cf;
        ff_sincos(d.omega[idx] * elapsed, sf, cf);
        const cx<T> p = mk<T>(cf, sf);
        auto ld = [](const double* q) { return mk<T>(ff_from_double(q[0]), ff_from_double(q[1])); };
        const cx<T> ap = cmul<T>(ld(Ap + 2 * idx), p);
        const cx<T> am = cmul<T>(ld(Am + 2 * idx), cconj<T>(p));
        const cx<T> a0 = ld(A0 + 2 * idx);
        const cx<T> uap = reinterpret_cast<const cx<T>*>(d.fUAp)[idx];
        const cx<T> vap = reinterpret_cast<const cx<T>*>(d.fVAp)[idx];
        const cx<T> wap = reinterpret_cast<const cx<T>*>(d.fWAp)[idx];
        const cx<T> ua0 = reinterpret_cast<const cx<T>*>(d.fUA0)[idx];
        const cx<T> va0 = reinterpret_cast<const cx<T>*>(d.fVA0)[idx];
        const T nap = reinterpret_cast<const T*>(d.fNAp)[idx], na0 = reinterpret_cast<const T*>(d.fNA0)[idx];
        cx<T> u = cadd<T>(cadd<T>(cmul<T>(uap, ap), cmul<T>(cconj<T>(uap), am)), cmul<T>(ua0, a0));
        cx<T> v = cadd<T>(cadd<T>(cmul<T>(vap, ap), cmul<T>(cconj<T>(vap), am)), cmul<T>(va0, a0));
        cx<T> ww = cadd<T>(cmul<T>(wap, ap), cmul<T>(wap, am));
        cx<T> n = mk<T>(ap.x * nap - am.x * nap + a0.x * na0, ap.y * nap - am.y * nap + a0.y * na0);
        if (flags & 1) { u = cconj<T>(u); v = cconj<T>(v); ww = cconj<T>(ww); n = cconj<T>(n); }
        if (flags & 2) { u.y = T(0); v.y = T(0); ww.y = T(0); n.y = T(0); }
        f[0] = u;
        f[1] = v;
        f[2] = ww;
        f[3] = n;
        return;
    }
    double s, c;
    sincos(d.omega[idx] * elapsed, &s, &c);
    const zd p{c, s};
    // evolveWaveVortexCoefficients + coefficientValueForField<0..3> (WVCoefficientFormulas.hpp:23-33)
    const zd ap = zmul(zload(Ap + 2 * idx), p);
    const zd am = zmul(zload(Am + 2 * idx), zconj(p));
    const zd a0 = zload(A0 + 2 * idx);
    const zd uap = zload(d.UAp + 2 * idx), vap = zload(d.VAp + 2 * idx), wap = zload(d.WAp + 2 * idx);
    const zd ua0 = zload(d.UA0 + 2 * idx), va0 = zload(d.VA0 + 2 * idx);
    const double nap = d.NAp[idx], na0 = d.NA0[idx];
    zd u = zadd(zadd(zmul(uap, ap), zmul(zconj(uap), am)), zmul(ua0, a0));
    zd v = zadd(zadd(zmul(vap, ap), zmul(zconj(vap), am)), zmul(va0, a0));
    zd ww = zadd(zmul(wap, ap), zmul(wap, am));
    zd n = zadd(zadd(zscale(ap, nap), zscale(am, -nap)), zscale(a0, na0));
    if (flags & 1) { u = zconj(u); v = zconj(v); ww = zconj(ww); n = zconj(n); }
    if (flags & 2) { u.im = 0.0; v.im = 0.0; ww.im = 0.0; n.im = 0.0; }
    f[0] = mk<T>(T(u.re), T(u.im));
    f[1] = mk<T>(T(v.re), T(v.im));
    f[2] = mk<T>(T(ww.re), T(ww.im));
    f[3] = mk<T>(T(n.re), T(n.im));
}

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256) k_vinv(DescDev d, const double* __restrict__ Ap, const double* __restrict__ Am,
                                             const double* __restrict__ A0, double elapsed, cx<T>* __restrict__ zspec,
                                             unsigned long long* __restrict__ maxSpeedBits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // fld[f][j][mode], f = u, v, w, eta (stored frame), working precision T
    cx<T>* fld = reinterpret_cast<cx<T>*>(smem_raw);
    const int Nj = d.Nj;
    const int m0 = blockIdx.x * kVinvModes;
    const int nm = min(kVinvModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        zspec += (size_t)member * d.Nz * d.positions;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && maxSpeedBits) maxSpeedBits[member] = 0ull;
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it / Nj, j = it - mi * Nj;
        cx<T> f[4];
        vinv_field_spectra<T>(d, Ap, Am, A0, elapsed, m0 + mi, j, f);
#pragma unroll
        for (int q = 0; q < 4; ++q) fld[(q * Nj + j) * kVinvModes + mi] = f[q];
    }
    __syncthreads();
    const int Zh = d.zHalf, Nz = d.Nz, P = d.positions;
    const T* Cc = reinterpret_cast<const T*>(d.Ccos);
    const T* Cs = reinterpret_cast<const T*>(d.Csin);
    const T* Ccm = reinterpret_cast<const T*>(d.CcosM);
    const T* Csm = reinterpret_cast<const T*>(d.CsinM);
    // channel layout: 0 U(cos u) 1 V(cos v) 2 W(sin w) 3 N(sin eta) then d/dz per flux target
    for (int it = threadIdx.x; it < nm * Zh; it += blockDim.x) {
        const int n = it / nm;
        const int mm = it - n * nm;
        const int mode = m0 + mm;
        // E (even j) and O (odd j) partial sums; channels U V W N Uz Vz Wz Nz
        T E[8][2], O[8][2];
#pragma unroll
        for (int a = 0; a < 8; ++a) { E[a][0] = T(0); E[a][1] = T(0); O[a][0] = T(0); O[a][1] = T(0); }
        const T* cc = Cc + n * Nj;
        const T* cs = Cs + n * Nj;
        const T* ccm = Ccm + n * Nj;
        const T* csm = Csm + n * Nj;
        auto accum = [&](T (&A)[8][2], int j) {
            const cx<T> u = fld[(0 * Nj + j) * kVinvModes + mm];
            const cx<T> v = fld[(1 * Nj + j) * kVinvModes + mm];
            const cx<T> w = fld[(2 * Nj + j) * kVinvModes + mm];
            const cx<T> e = fld[(3 * Nj + j) * kVinvModes + mm];
            const T a = cc[j], b = cs[j];
            A[0][0] += a * u.x; A[0][1] += a * u.y;
            A[1][0] += a * v.x; A[1][1] += a * v.y;
            A[2][0] += b * w.x; A[2][1] += b * w.y;
            A[3][0] += b * e.x; A[3][1] += b * e.y;
            if (FLUX) {
                const T am = ccm[j], bm = csm[j];
                A[4][0] += bm * u.x; A[4][1] += bm * u.y;
                A[5][0] += bm * v.x; A[5][1] += bm * v.y;
                A[6][0] += am * w.x; A[6][1] += am * w.y;
                A[7][0] += am * e.x; A[7][1] += am * e.y;
            }
        };
        int j = 0;
        for (; j + 1 < Nj; j += 2) { accum(E, j); accum(O, j + 1); }
        if (j < Nj) accum(E, j);
        const int pos = d.modePos[mode];
        const int cpos = d.modeCompPos[mode];
        const int n2 = Nz - 1 - n;
        auto put = [&](int ch, const T* Ec, const T* Oc, bool sine) {
            // cos family: out[n] = E+O, out[Nz-1-n] = E-O ; sin family: out[Nz-1-n] = O-E
            cx<T>* base = zspec + (size_t)ch * d.zTotal * P;
            const cx<T> lo = mk<T>(Ec[0] + Oc[0], Ec[1] + Oc[1]);
            base[(size_t)n * P + pos] = lo;
            if (cpos >= 0) base[(size_t)n * P + cpos] = mk<T>(lo.x, -lo.y);
            if (n2 != n) {
                const cx<T> hi = sine ? mk<T>(Oc[0] - Ec[0], Oc[1] - Ec[1]) : mk<T>(Ec[0] - Oc[0], Ec[1] - Oc[1]);
                base[(size_t)n2 * P + pos] = hi;
                if (cpos >= 0) base[(size_t)n2 * P + cpos] = mk<T>(hi.x, -hi.y);
            }
        };
        put(0, E[0], O[0], false);
        put(1, E[1], O[1], false);
        put(2, E[2], O[2], true);
        put(3, E[3], O[3], true);
        if (FLUX) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (t < d.nt) {
                    const int q = d.tq[t];
                    if (q == 0) put(4 + t, E[4], O[4], true);
                    else if (q == 1) put(4 + t, E[5], O[5], true);
                    else if (q == 2) put(4 + t, E[6], O[6], false);
                    else put(4 + t, E[7], O[7], false);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// vinv_family: value and z derivative of the F (FFAMILY) or G field family of
// (Apm, A0) per retained column (fieldFamilyDerivativeSpectrum,
// WVCoefficientFormulas.hpp:60-73): value = Apm waveScale + A0 geostrophicScale
// in the stored frame, F values through the cosine matrix and their -m z
// derivative through CsinM; G values through the sine matrix and their +m z
// derivative through CcosM -> zspec[0 | 1][z][pos].

template <typename T, bool FFAMILY>
__global__ void __launch_bounds__(256) k_vinv_family(DescDev d, const double* __restrict__ Apm, const double* __restrict__ A0,
                                                    cx<T>* __restrict__ zspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* fld = reinterpret_cast<cx<T>*>(smem_raw);  // [Nj][modes]
    const int Nj = d.Nj;
    const int m0 = blockIdx.x * kVinvModes;
    const int nm = min(kVinvModes, d.Nkl - m0);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it / Nj, j = it - mi * Nj;
        const int mode = m0 + mi;
        const int w = d.modeWV[mode];
        const unsigned char flags = d.modeFlags[mode];
        const int idx = j + Nj * w;
        const double ws = FFAMILY ? d.fWaveScale[idx] : d.gWaveScale[j];
        const double gs = FFAMILY ? d.Fg[j] : d.Gg[j];
        const zd v = zadd(zscale(zload(Apm + 2 * idx), ws), zscale(zload(A0 + 2 * idx), gs));
        double re = v.re, im = v.im;
        if (flags & 1) im = -im;
        if (flags & 2) im = 0.0;
        fld[j * kVinvModes + mi] = mk<T>(T(re), T(im));
    }
    __syncthreads();
    const int Zh = d.zHalf, Nz = d.Nz, P = d.positions;
    const T* Cv = reinterpret_cast<const T*>(FFAMILY ? d.Ccos : d.Csin);
    const T* Cz = reinterpret_cast<const T*>(FFAMILY ? d.CsinM : d.CcosM);
    for (int it = threadIdx.x; it < nm * Zh; it += blockDim.x) {
        const int n = it / nm, mm = it - n * nm;
        const int mode = m0 + mm;
        T E[2][2] = {{T(0), T(0)}, {T(0), T(0)}}, O[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
        for (int j = 0; j < Nj; ++j) {
            const cx<T> v = fld[j * kVinvModes + mm];
            const T a = Cv[n * Nj + j], b = Cz[n * Nj + j];
            T (&A)[2][2] = (j & 1) ? O : E;
            A[0][0] += a * v.x; A[0][1] += a * v.y;
            A[1][0] += b * v.x; A[1][1] += b * v.y;
        }
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const int n2 = Nz - 1 - n;
        for (int ch = 0; ch < 2; ++ch) {
            // cosine family: out[n2] = E - O; sine family: O - E
            const bool sine = FFAMILY ? ch == 1 : ch == 0;
            cx<T>* base = zspec + (size_t)ch * d.zTotal * P;
            const cx<T> lo = mk<T>(E[ch][0] + O[ch][0], E[ch][1] + O[ch][1]);
            base[(size_t)n * P + pos] = lo;
            if (cpos >= 0) base[(size_t)n * P + cpos] = mk<T>(lo.x, -lo.y);
            if (n2 != n) {
                const cx<T> hi = sine ? mk<T>(O[ch][0] - E[ch][0], O[ch][1] - E[ch][1]) : mk<T>(E[ch][0] - O[ch][0], E[ch][1] - O[ch][1]);
                base[(size_t)n2 * P + pos] = hi;
                if (cpos >= 0) base[(size_t)n2 * P + cpos] = mk<T>(hi.x, -hi.y);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// yinv: inverse FFT along y for kx columns [kx0, kx0+G) of plane z.
// Output channel oc reads input channel src[oc]; if mulL[oc], multiplies by i*l.

constexpr int kYG = 4;

struct YInvMap {
    int nOut;
    int src[16];
    int mulL[16];
};

// Output channel c of k_yfwd_pair(_w) = FFT_y(srcA[c]) + (-i l) FFT_y(srcB[c]) (srcB < 0: none).
struct YFwdPairMap {
    int nOut;
    int srcA[8];
    int srcB[8];
};

template <typename T>
__global__ void __launch_bounds__(256) k_yinv(DescDev d, YInvMap map, const cx<T>* __restrict__ zspec, int nInCh,
                                             cx<T>* __restrict__ yspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, P = d.positions, KX = d.kxColumns;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* bufA = tw + Ny;
    cx<T>* bufB = bufA + kYG * Ny;
    const int kx0 = blockIdx.x * kYG;
    const int z = blockIdx.y;
    const int g = min(kYG, KX - kx0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < Ny; i += blockDim.x) tw[i] = twg[i];
    (void)nInCh;
    for (int oc = 0; oc < map.nOut; ++oc) {
        for (int i = threadIdx.x; i < kYG * Ny; i += blockDim.x) bufA[i] = mk<T>(T(0), T(0));
        __syncthreads();
        const cx<T>* in = zspec + ((size_t)map.src[oc] * d.zTotal + z) * P;
        const int pBeg = d.colStart[kx0], pEnd = d.colStart[kx0 + g];
        for (int p = pBeg + threadIdx.x; p < pEnd; p += blockDim.x) {
            // column of p
            int gi = 0;
            while (gi + 1 < g && p >= d.colStart[kx0 + gi + 1]) ++gi;
            const int ky = d.posKy[p];
            cx<T> v = in[p];
            if (map.mulL[oc]) {
                const T l = row_l<T>(d)[ky];
                v = mk<T>(-l * v.y, l * v.x);
            }
            bufA[gi * Ny + ky] = v;
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, true>(bufA, bufB, d.fy, g, Ny, tw);
        cx<T>* out = yspec + (((size_t)z * map.nOut + oc) * Ny) * KX;
        for (int i = threadIdx.x; i < g * Ny; i += blockDim.x) {
            const int y = i / g, gi = i - y * g;
            out[(size_t)y * KX + kx0 + gi] = res[gi * Ny + y];
        }
        __syncthreads();
        if (res != bufA) {
            // keep bufA/bufB roles fixed for the next channel
        }
    }
}

// ---------------------------------------------------------------------------
// Real transforms along x, one real row per complex line.  For even Nx a row
// of Nx reals is one complex line of Nx/2 (the standard split of even and odd
// samples), so each row's rounding stays relative to its own magnitude.

// Half-spectrum value at 0 <= k <= Nx/2 (zero for k >= KX), optionally times
// i*k_row; imaginary parts at k = 0 and k = Nx/2 are dropped (c2r semantics).
template <typename T>
__device__ __forceinline__ cx<T> half_at(const cx<T>* h, int k, int KX, int Nx, const T* rowK, bool useK) {
    if (k >= KX) return mk<T>(T(0), T(0));
    cx<T> v = h[k];
    if (k == 0 || 2 * k == Nx) v.y = T(0);
    if (useK) {
        const T kk = rowK[k];
        v = mk<T>(-kk * v.y, kk * v.x);
    }
    return v;
}

// Entry k of the complex line whose inverse FFT yields the real row.
template <typename T>
__device__ __forceinline__ cx<T> c2r_line_entry(const DescDev& d, const cx<T>* h, int k, bool useK, const cx<T>* twN) {
    const int Nx = d.Nx, KX = d.kxColumns;
    if (d.xEven) {
        const int M = Nx >> 1;
        const cx<T> a = half_at<T>(h, k, KX, Nx, row_k<T>(d), useK);
        const cx<T> b = cconj<T>(half_at<T>(h, M - k, KX, Nx, row_k<T>(d), useK));
        const cx<T> e = cadd<T>(a, b);
        const cx<T> o = cmul<T>(csub<T>(a, b), cconj<T>(twN[k]));  // * exp(+2 pi i k/Nx)
        return mk<T>(e.x - o.y, e.y + o.x);                        // e + i o
    }
    if (2 * k <= Nx) return half_at<T>(h, k, KX, Nx, row_k<T>(d), useK);
    return cconj<T>(half_at<T>(h, Nx - k, KX, Nx, row_k<T>(d), useK));
}

// Real sample x of the row from the inverse-transformed line.
template <typename T>
__device__ __forceinline__ T c2r_sample(const DescDev& d, const cx<T>* line, int x) {
    if (d.xEven) { const cx<T> v = line[x >> 1]; return (x & 1) ? v.y : v.x; }
    return line[x].x;
}

// Entry n of the complex line whose forward FFT gives the row's spectrum.
template <typename T>
__device__ __forceinline__ cx<T> r2c_line_entry(const DescDev& d, const T* row, int n) {
    if (d.xEven) return mk<T>(row[2 * n], row[2 * n + 1]);
    return mk<T>(row[n], T(0));
}

// Spectrum value at k < KX from the forward-transformed line.
template <typename T>
__device__ __forceinline__ cx<T> r2c_value(const DescDev& d, const cx<T>* line, int k, const cx<T>* twN) {
    if (d.xEven) {
        const int M = d.Nx >> 1;
        const int km = k >= M ? k - M : k;  // k mod M for 0 <= k < 2M
        const cx<T> zk = line[km];
        const cx<T> zn = cconj<T>(line[km == 0 ? 0 : M - km]);
        const cx<T> e = mk<T>(T(0.5) * (zk.x + zn.x), T(0.5) * (zk.y + zn.y));
        const cx<T> df = csub<T>(zk, zn);
        const cx<T> o = mk<T>(T(0.5) * df.y, T(-0.5) * df.x);  // (zk - zn) / (2i)
        return cadd<T>(e, cmul<T>(twN[k], o));
    }
    return line[k];
}

// ---------------------------------------------------------------------------
// xflux: one CTA per (y, z) row.

// physOut, when given, receives the real rows [z][nReal][y][Nx] for the adjoint.
// advOut, when given, receives the advecting (u, v, w) as doubles [3][z][y][Nx];
// advIn, when given, replaces them (nonlinearFlux With/Using AdvectionFields).
template <typename T>
__global__ void __launch_bounds__(256) k_xflux(DescDev d, const cx<T>* __restrict__ yspec, cx<T>* __restrict__ pspec,
                                              unsigned long long* __restrict__ maxSpeedBits, T* __restrict__ physOut,
                                              double* __restrict__ advOut, const double* __restrict__ advIn) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, KX = d.kxColumns, nt = d.nt, L = d.xLen;
    const int nIn = 4 + 2 * nt;          // U V W N, q_y..., q_z...
    const int nReal = 3 + 3 * nt;        // U V W, then (q_x, q_y, q_z) per target
    const bool lPow2 = (L & (L - 1)) == 0;
    const int lShift = __ffs(L) - 1;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);  // [L]
    cx<T>* twN = tw + L;                              // [Nx]
    cx<T>* bufA = twN + Nx;                           // [8][L]
    cx<T>* bufB = bufA + 8 * L;
    T* phys = reinterpret_cast<T*>(bufB + 8 * L);    // U, V, W [3][Nx], then S_q [nt][Nx]
    T* S = phys + 3 * Nx;
    // the row's channel spectra are read from L2 where the lines are built (no
    // staging copy: the smaller footprint fits one more CTA per SM)
    const cx<T>* yrow = yspec + ((size_t)z * nIn * Ny + y) * KX;
    const size_t cstride = (size_t)Ny * KX;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) twN[i] = twgN[i];
    __syncthreads();
    // real row r -> (input channel, times i*k)
    auto rowSrc = [&](int r, int& ch, bool& useK) {
        if (r < 3) { ch = r; useK = false; return; }
        const int t = (r - 3) / 3, kind = (r - 3) % 3;
        const int q = d.tq[t];
        if (kind == 0) { ch = q; useK = true; }          // q_x = i k q   (q indexes U,V,W,N)
        else if (kind == 1) { ch = 4 + t; useK = false; } // q_y
        else { ch = 4 + nt + t; useK = false; }           // q_z
    };
    const size_t R3 = (size_t)Nx * Ny * d.Nz;
    // Rows in batches of 8 lines.  U, V, W stay in shared memory; each derivative
    // row is folded into its target's product as soon as it is transformed,
    // S_q = -(u q_x + v q_y + w q_z) accumulated in that order (one thread per x
    // walks a batch's rows in order, so the order is the same for every x).
    for (int rb = 0; rb < nReal; rb += 8) {
        const int nr = min(8, nReal - rb);
        for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
            const int li = lPow2 ? i >> lShift : i / L, k = i - li * L;
            int ch; bool useK;
            rowSrc(rb + li, ch, useK);
            bufA[li * L + k] = c2r_line_entry<T>(d, yrow + ch * cstride, k, useK, twN);
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, true>(bufA, bufB, d.fx, nr, L, tw);
        if (rb == 0) {
            for (int i = threadIdx.x; i < 3 * Nx; i += blockDim.x) {
                const int c = i / Nx, x = i - c * Nx;
                const size_t g = (size_t)c * R3 + ((size_t)z * Ny + y) * Nx + x;
                T v = c2r_sample<T>(d, res + c * L, x);
                if (advIn) v = T(advIn[g]);
                else if (advOut) advOut[g] = double(v);
                phys[i] = v;
            }
            __syncthreads();
        }
        for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
            for (int li = (rb == 0 ? 3 : 0); li < nr; ++li) {
                const int r = rb + li;
                const T v = c2r_sample<T>(d, res + li * L, x);
                if (physOut) physOut[(((size_t)z * nReal + r) * Ny + y) * Nx + x] = v;
                const int t = (r - 3) / 3, kind = (r - 3) % 3;
                const T p = phys[kind * Nx + x] * v;
                S[t * Nx + x] = kind == 0 ? p : S[t * Nx + x] + p;
            }
        }
        __syncthreads();
    }
    if (physOut)
        for (int i = threadIdx.x; i < 3 * Nx; i += blockDim.x) {
            const int r = i / Nx, x = i - r * Nx;
            physOut[(((size_t)z * nReal + r) * Ny + y) * Nx + x] = phys[i];
        }
    // max |u_h| (only when a consumer asked for it): max of u^2 + v^2, one sqrt
    // at the end -- sqrt is correctly rounded and monotone, so this equals the
    // max over points of sqrt(u^2 + v^2)
    const bool wantSpeed = maxSpeedBits != nullptr;
    double vmax2 = 0.0;
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        for (int t = 0; t < nt; ++t) S[t * Nx + x] = -S[t * Nx + x];
        if (wantSpeed) {
            const T U = phys[x], V = phys[Nx + x];
            vmax2 = fmax(vmax2, double(U) * double(U) + double(V) * double(V));
        }
    }
    __syncthreads();  // S complete before the forward real transforms read it
    if (wantSpeed) {
        for (int o = 16; o > 0; o >>= 1) vmax2 = fmax(vmax2, __shfl_xor_sync(0xffffffffu, vmax2, o));
        __shared__ double red[32];
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmax(m, red[i]);
            atomicMax(maxSpeedBits + z / d.Nz, (unsigned long long)__double_as_longlong(sqrt(m)));
        }
    }
    // forward real transform of each S_q
    for (int i = threadIdx.x; i < nt * L; i += blockDim.x) {
        const int t = lPow2 ? i >> lShift : i / L, n = i - t * L;
        bufB[t * L + n] = r2c_line_entry<T>(d, S + t * Nx, n);
    }
    __syncthreads();
    cx<T>* res = fft_lines<T, false>(bufB, bufA, d.fx, nt, L, tw);
    for (int i = threadIdx.x; i < nt * KX; i += blockDim.x) {
        const int t = i / KX, k = i - t * KX;
        pspec[(((size_t)z * nt + t) * Ny + y) * KX + k] = r2c_value<T>(d, res + t * L, k, twN);
    }
}

// ---------------------------------------------------------------------------
// xc2r_fields: c2r of nch channel spectra to the real rows of a field bundle
// fields[ch][z][y][x] (x fastest) -- transformWaveVortexToUVWEta output.

template <typename T>
__global__ void __launch_bounds__(256) k_xc2r_fields(DescDev d, const cx<T>* __restrict__ yspec, int nch,
                                                    double* __restrict__ fields) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, Nz = d.Nz, KX = d.kxColumns, L = d.xLen;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* twN = tw + L;
    cx<T>* spec = twN + Nx;
    cx<T>* bufA = spec + nch * KX;
    cx<T>* bufB = bufA + 4 * L;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) twN[i] = twgN[i];
    for (int i = threadIdx.x; i < nch * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        spec[i] = yspec[(((size_t)z * nch + c) * Ny + y) * KX + k];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nch * L; i += blockDim.x) {
        const int li = i / L, k = i - li * L;
        bufA[li * L + k] = c2r_line_entry<T>(d, spec + li * KX, k, ((d.c2rUseK >> li) & 1) != 0, twN);
    }
    __syncthreads();
    cx<T>* res = fft_lines<T, true>(bufA, bufB, d.fx, nch, L, tw);
    const size_t R = (size_t)Nx * Ny * Nz;
    for (int i = threadIdx.x; i < nch * Nx; i += blockDim.x) {
        const int li = i / Nx, x = i - li * Nx;
        fields[(size_t)li * R + ((size_t)z * Ny + y) * Nx + x] = double(c2r_sample<T>(d, res + li * L, x));
    }
}

// xr2c_fields: r2c along x of field rows -> pspec[z][ch][y][kx] (kx < KX).
template <typename T>
__global__ void __launch_bounds__(256) k_xr2c_fields(DescDev d, const double* __restrict__ fields, int nch,
                                                    cx<T>* __restrict__ pspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, Nz = d.Nz, KX = d.kxColumns, L = d.xLen;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* twN = tw + L;
    cx<T>* bufA = twN + Nx;
    cx<T>* bufB = bufA + 4 * L;
    T* row = reinterpret_cast<T*>(bufB + 4 * L);  // [nch][Nx]
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) twN[i] = twgN[i];
    const size_t R = (size_t)Nx * Ny * Nz;
    for (int i = threadIdx.x; i < nch * Nx; i += blockDim.x) {
        const int c = i / Nx, x = i - c * Nx;
        row[c * Nx + x] = T(fields[(size_t)c * R + ((size_t)z * Ny + y) * Nx + x]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nch * L; i += blockDim.x) {
        const int c = i / L, n = i - c * L;
        bufA[c * L + n] = r2c_line_entry<T>(d, row + c * Nx, n);
    }
    __syncthreads();
    cx<T>* res = fft_lines<T, false>(bufA, bufB, d.fx, nch, L, tw);
    for (int i = threadIdx.x; i < nch * KX; i += blockDim.x) {
        const int t = i / KX, k = i - t * KX;
        pspec[(((size_t)z * nch + t) * Ny + y) * KX + k] = r2c_value<T>(d, res + t * L, k, twN);
    }
}

// ---------------------------------------------------------------------------
// yfwd: forward FFT along y for kx columns [kx0, kx0+G) of plane z, channel c;
// gathered to the active rows: fspec[c][z][pos].

template <typename T>
__global__ void __launch_bounds__(256) k_yfwd(DescDev d, const cx<T>* __restrict__ pspec, int nch, cx<T>* __restrict__ fspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, P = d.positions, KX = d.kxColumns;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* bufA = tw + Ny;
    cx<T>* bufB = bufA + kYG * Ny;
    const int kx0 = blockIdx.x * kYG;
    const int z = blockIdx.y;
    const int c = blockIdx.z;
    const int g = min(kYG, KX - kx0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < Ny; i += blockDim.x) tw[i] = twg[i];
    const cx<T>* in = pspec + (((size_t)z * nch + c) * Ny) * KX;
    for (int i = threadIdx.x; i < g * Ny; i += blockDim.x) {
        const int y = i / g, gi = i - y * g;
        bufA[gi * Ny + y] = in[(size_t)y * KX + kx0 + gi];
    }
    __syncthreads();
    cx<T>* res = fft_lines<T, false>(bufA, bufB, d.fy, g, Ny, tw);
    cx<T>* out = fspec + ((size_t)c * d.zTotal + z) * P;
    const int pBeg = d.colStart[kx0], pEnd = d.colStart[kx0 + g];
    for (int p = pBeg + threadIdx.x; p < pEnd; p += blockDim.x) {
        int gi = 0;
        while (gi + 1 < g && p >= d.colStart[kx0 + gi + 1]) ++gi;
        out[p] = res[gi * Ny + d.posKy[p]];
    }
}

// ---------------------------------------------------------------------------
// vfwd: forward vertical contraction and projection.
//  FLUX:  accumulates the nonlinear flux of every target (projectFluxTargetMode)
//         and, when damping != null, adds A * (maxSpeed * damping).
//  !FLUX: forward transform (projectNonhydrostaticMode / projectHydrostaticMode).

constexpr int kVfwdModes = 8;

// MIXED flux projection of one (mode, j): the folded FP32 map (fProj: Cu, Cv,
// Cw complex, Du, Dv, Dn, Npm, B) of the target spectra ch[q] = (u, v, w, eta)
// -> cp, cm, f0, an FP32 phase after FP64 angle reduction, FP64 adaptive
// damping and FP64 stores (projectFluxTargetMode, kernel.cpp:396-431).
__device__ __forceinline__ void mixed_project_store(const DescDev& d, int idx, int w, int j, const float2 (&ch)[4],
                                                    double elapsed, double maxSpeed, int applyDamping,
                                                    const double* __restrict__ Ap, const double* __restrict__ Am,
                                                    const double* __restrict__ A0, double* __restrict__ Fp,
                                                    double* __restrict__ Fm, double* __restrict__ F0) {
    const float2 U = ch[0], V = ch[1], Wc = ch[2], N = ch[3];
    const float4* pj = reinterpret_cast<const float4*>(d.fProj + 12 * (size_t)idx);
    const float4 p0 = pj[0], p1 = pj[1], p2 = pj[2];
    const float f0r = -p1.z * U.y - p1.w * V.y + p2.x * N.x;
    const float f0i = p1.z * U.x + p1.w * V.x + p2.x * N.y;
    float cpr, cpi, cmr, cmi;
    if (w == 0) {
        const float sc = float(d.inertialScale[j]);
        cpr = sc * (U.x + V.y);
        cpi = sc * (U.y - V.x);
        cmr = cpr;
        cmi = -cpi;
    } else {
        const float wr = p0.x * U.x - p0.y * U.y + p0.z * V.x - p0.w * V.y + p1.x * Wc.x - p1.y * Wc.y;
        const float wi = p0.x * U.y + p0.y * U.x + p0.z * V.y + p0.w * V.x + p1.x * Wc.y + p1.y * Wc.x;
        const float br = p2.y * N.x - p2.z * f0r, bi = p2.y * N.y - p2.z * f0i;
        cpr = wr + br; cpi = wi + bi; cmr = wr - br; cmi = wi - bi;
    }
    const double ang = d.omega[idx] * elapsed;
    const double red = ang - 6.283185307179586476925 * rint(ang * 0.15915494309189533577);
    float sn, cs;
    sincosf(float(red), &sn, &cs);
    zd fp{double(cpr * cs + cpi * sn), double(cpi * cs - cpr * sn)};   // (cp) * conj(p)
    zd fm{double(cmr * cs - cmi * sn), double(cmr * sn + cmi * cs)};   // (cm) * p
    zd f0{double(f0r), double(f0i)};
    if (applyDamping) {
        const double sd = __dmul_rn(maxSpeed, d.damping[idx]);
        fp = zadd(fp, zscale(zload(Ap + 2 * idx), sd));
        fm = zadd(fm, zscale(zload(Am + 2 * idx), sd));
        f0 = zadd(f0, zscale(zload(A0 + 2 * idx), sd));
    }
    zstore(Fp + 2 * idx, fp);
    zstore(Fm + 2 * idx, fm);
    zstore(F0 + 2 * idx, f0);
}

template <typename T>
struct cx2t { cx<T> p, q; };

// Projection of one (mode, j) of the forward transform: vr / vi hold the
// transformed channels (canonical frame).  FLUX: the flux of every target with
// the phase rotation and optional adaptive damping (projectFluxTargetMode,
// kernel.cpp:396-431); !FLUX: the forward transform (projectNonhydrostaticMode
// / projectHydrostaticMode, kernel.cpp:299-370).  Pointers are the member's.
template <typename T, bool FLUX>
__device__ __forceinline__ void vfwd_project(const DescDev& d, int w, int j, const T (&vr)[4], const T (&vi)[4], int nch,
                                             double elapsed, double maxSpeed, int applyDamping,
                                             const double* __restrict__ Ap, const double* __restrict__ Am,
                                             const double* __restrict__ A0, double* __restrict__ Fp,
                                             double* __restrict__ Fm, double* __restrict__ F0) {
    const int Nj = d.Nj;
    const int idx = j + Nj * w;
    if constexpr (FLUX && std::is_same<T, ff>::value) {
        // FP32X2 flux: the folded projection of the mixed form with paired-FP32
        // coefficients (d.fProj holds 12 ff per (mode, j)) and an FP64 phase.
        cx<T> ch[4] = {mk<T>(T(0), T(0)), mk<T>(T(0), T(0)), mk<T>(T(0), T(0)), mk<T>(T(0), T(0))};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            ch[d.tq[c]] = mk<T>(vr[c], vi[c]);
        }
        const cx<T> U = ch[0], V = ch[1], Wc = ch[2], N = ch[3];
        const T* pj = reinterpret_cast<const T*>(d.fProj) + 12 * (size_t)idx;
        const T f0r = -pj[6] * U.y - pj[7] * V.y + pj[8] * N.x;
        const T f0i = pj[6] * U.x + pj[7] * V.x + pj[8] * N.y;
        T cpr, cpi, cmr, cmi;
        if (w == 0) {
            const T sc = T(d.inertialScale[j]);
            cpr = sc * (U.x + V.y);
            cpi = sc * (U.y - V.x);
            cmr = cpr;
            cmi = -cpi;
        } else {
            const T wr = pj[0] * U.x - pj[1] * U.y + pj[2] * V.x - pj[3] * V.y + pj[4] * Wc.x - pj[5] * Wc.y;
            const T wi = pj[0] * U.y + pj[1] * U.x + pj[2] * V.y + pj[3] * V.x + pj[4] * Wc.y + pj[5] * Wc.x;
            const T br = pj[9] * N.x - pj[10] * f0r, bi = pj[9] * N.y - pj[10] * f0i;
            cpr = wr + br; cpi = wi + bi; cmr = wr - br; cmi = wi - bi;
        }
        T sn, cs;
        ff_sincos(d.omega[idx] * elapsed, sn, cs);
        zd fp{double(cpr * cs + cpi * sn), double(cpi * cs - cpr * sn)};   // (cp) * conj(p)
        zd fm{double(cmr * cs - cmi * sn), double(cmr * sn + cmi * cs)};   // (cm) * p
        zd f0{double(f0r), double(f0i)};
        if (applyDamping) {
            const double sdmp = __dmul_rn(maxSpeed, d.damping[idx]);
            fp = zadd(fp, zscale(zload(Ap + 2 * idx), sdmp));
            fm = zadd(fm, zscale(zload(Am + 2 * idx), sdmp));
            f0 = zadd(f0, zscale(zload(A0 + 2 * idx), sdmp));
        }
        zstore(Fp + 2 * idx, fp);
        zstore(Fm + 2 * idx, fm);
        zstore(F0 + 2 * idx, f0);
    } else if constexpr (FLUX && sizeof(T) == 4) {
        // MIXED flux: projection with the folded FP32 coefficients
        float2 ch[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            ch[d.tq[c]] = make_float2(float(vr[c]), float(vi[c]));
        }
        mixed_project_store(d, idx, w, j, ch, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
    } else {
    zd val[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) val[c] = zd{double(vr[c]), double(vi[c])};
const double k = d.k[w], l = d.l[w];
    double s, cph;
    sincos(d.omega[idx] * elapsed, &s, &cph);
    const zd p{cph, s};
    if (FLUX) {
        // Contributions of every target are summed first and rotated to the
        // reference time once: sum_q c_q conj(p) = (sum_q c_q) conj(p).
        // Per-target formulas of projectFluxTargetMode (kernel.cpp:396-431);
        // contraction into FMA is allowed here.
        const double vort = d.A0FromVorticity[idx], buoyF = d.A0FromBuoyancy[idx];
        const double na0 = d.NA0[idx], apmn = d.ApmN[idx];
        double cpr = 0.0, cpi = 0.0, cmr = 0.0, cmi = 0.0, f0r = 0.0, f0i = 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            const int q = d.tq[c];
            const zd v = val[c];
            double ar = 0.0, ai = 0.0;  // A0 contribution
            if (q == 0) { ar = (v.im * l) * vort; ai = (-v.re * l) * vort; }
            if (q == 1) { ar = (-v.im * k) * vort; ai = (v.re * k) * vort; }
            if (q == 3) { ar = v.re * buoyF; ai = v.im * buoyF; }
            double br = -ar * na0, bi = -ai * na0;  // buoyancy value
            if (q == 3) { br += v.re; bi += v.im; }
            br *= apmn; bi *= apmn;
            double wr = 0.0, wi = 0.0;  // wave contribution
            if (d.hydrostatic) {
                const zd apmd = zload(d.ApmD + 2 * idx);
                double xr = 0.0, xi = 0.0;  // value * i*(k or l)
                if (q == 0) { xr = -v.im * k; xi = v.re * k; }
                if (q == 1) { xr = -v.im * l; xi = v.re * l; }
                wr = xr * apmd.re - xi * apmd.im;
                wi = xr * apmd.im + xi * apmd.re;
            } else {
                if (q == 0) { const double sc = d.cosAlpha[w] * d.ApmDScaled[idx]; wr = v.re * sc; wi = v.im * sc; }
                if (q == 1) { const double sc = d.sinAlpha[w] * d.ApmDScaled[idx]; wr = v.re * sc; wi = v.im * sc; }
                if (q == 2) { const double sc = (d.Kh[w] / 2.0) * d.apmWPrefactor[j]; wr = -v.im * sc; wi = v.re * sc; }
            }
            double pr = wr + br, pi = wi + bi, mr = wr - br, mi = wi - bi;
            if (w == 0) {
                const double sc = d.inertialScale[j];
                pr = 0.0; pi = 0.0;
                if (q == 0) { pr = v.re * sc; pi = v.im * sc; }
                if (q == 1) { pr = v.im * sc; pi = -v.re * sc; }
                mr = pr; mi = -pi;
            }
            cpr += pr; cpi += pi; cmr += mr; cmi += mi; f0r += ar; f0i += ai;
        }
        zd fp{cpr * p.re + cpi * p.im, cpi * p.re - cpr * p.im};   // (cp) * conj(p)
        zd fm{cmr * p.re - cmi * p.im, cmr * p.im + cmi * p.re};   // (cm) * p
        zd f0{f0r, f0i};
        if (applyDamping) {
            const double sd = __dmul_rn(maxSpeed, d.damping[idx]);
            fp = zadd(fp, zscale(zload(Ap + 2 * idx), sd));
            fm = zadd(fm, zscale(zload(Am + 2 * idx), sd));
            f0 = zadd(f0, zscale(zload(A0 + 2 * idx), sd));
        }
        zstore(Fp + 2 * idx, fp);
        zstore(Fm + 2 * idx, fm);
        zstore(F0 + 2 * idx, f0);
    } else {
        const zd U = val[0], V = val[1];
        const zd W = d.hydrostatic ? zd{0.0, 0.0} : val[2];
        const zd N = d.hydrostatic ? val[2] : val[3];
        const zd vort = zsub(zmul(V, zd{0.0, k}), zmul(U, zd{0.0, l}));
        const zd a0 = zadd(zscale(vort, d.A0FromVorticity[idx]), zscale(N, d.A0FromBuoyancy[idx]));
        zd cp, cm;
        if (w == 0) {
            cp = zscale(zsub(U, zmul(V, zd{0.0, 1.0})), d.inertialScale[j]);
            cm = zconj(cp);
        } else {
            const zd buoy = zscale(zsub(N, zscale(a0, d.NA0[idx])), d.ApmN[idx]);
            zd wave;
            if (d.hydrostatic) {
                const zd div = zadd(zmul(U, zd{0.0, k}), zmul(V, zd{0.0, l}));
                wave = zmul(zload(d.ApmD + 2 * idx), div);
            } else {
                const zd delta = zscale(zadd(zscale(U, d.cosAlpha[w]), zscale(V, d.sinAlpha[w])), d.ApmDScaled[idx]);
                const zd wbar = zmul(zd{0.0, __dmul_rn(d.Kh[w] / 2.0, d.apmWPrefactor[j])}, W);
                wave = zadd(delta, wbar);
            }
            cp = zadd(wave, buoy);
            cm = zsub(wave, buoy);
        }
        zstore(Fp + 2 * idx, zmul(cp, zconj(p)));
        zstore(Fm + 2 * idx, zmul(cm, p));
        zstore(F0 + 2 * idx, a0);
    }
    }  // FP64 projection
}

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256, VertOcc<T>::value) k_vfwd(DescDev d, const cx<T>* __restrict__ fspec, int nch, double elapsed,
                                             const double* __restrict__ Ap, const double* __restrict__ Am,
                                             const double* __restrict__ A0, const unsigned long long* __restrict__ maxSpeedBits,
                                             int applyDamping, double* __restrict__ Fp, double* __restrict__ Fm,
                                             double* __restrict__ F0) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions;
    const int m0 = blockIdx.x * kVfwdModes;
    const int nm = min(kVfwdModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        if (Ap) { Ap += o; Am += o; A0 += o; }
        Fp += o; Fm += o; F0 += o;
        fspec += (size_t)member * Nz * P;
        if (maxSpeedBits) maxSpeedBits += member;
    }
    // folded columns pq[c][n][mode] = (S_n + S_{Nz-1-n}, S_n - S_{Nz-1-n})
    cx2t<T>* pq = reinterpret_cast<cx2t<T>*>(smem_raw);
    for (int it = threadIdx.x; it < nch * Zh * nm; it += blockDim.x) {
        const int mm = it % nm;
        const int rest = it / nm;
        const int n = rest % Zh, c = rest / Zh;
        const int pos = d.modePos[m0 + mm];
        const cx<T>* col = fspec + (size_t)c * d.zTotal * P + pos;
        const cx<T> a = col[(size_t)n * P];
        const int n2 = Nz - 1 - n;
        cx2t<T> v;
        if (n2 == n) {
            v.p = a; v.q = a;
        } else {
            const cx<T> b = col[(size_t)n2 * P];
            v.p = cadd<T>(a, b); v.q = csub<T>(a, b);
        }
        pq[(c * Zh + n) * kVfwdModes + mm] = v;
    }
    __syncthreads();
    double maxSpeed = 0.0;
    if (FLUX && applyDamping) maxSpeed = __longlong_as_double((long long)*maxSpeedBits);
    const T* Fc = reinterpret_cast<const T*>(d.Fcos);
    const T* Fs = reinterpret_cast<const T*>(d.Fsin);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mm = it % nm, j = it / nm;
        const int mode = m0 + mm;
        const int w = d.modeWV[mode];
        const bool conj = d.modeFlags[mode] & 1;
        const bool evenJ = (j & 1) == 0;
        const T* fc = Fc + (size_t)j * Zh;
        const T* fs = Fs + (size_t)j * Zh;
        // forward vertical transform of each channel (stored frame -> canonical)
        T vr[4] = {T(0), T(0), T(0), T(0)}, vi[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            int q;
            if (FLUX) q = d.tq[c];
            else q = (d.hydrostatic && c == 2) ? 3 : c;
            const bool cosine = q < 2;
            const T* F = cosine ? fc : fs;
            const bool useP = cosine ? evenJ : !evenJ;
            T re = T(0), im = T(0);
            const cx2t<T>* col = pq + (size_t)c * Zh * kVfwdModes + mm;
            for (int n = 0; n < Zh; ++n) {
                const cx2t<T> v = col[n * kVfwdModes];
                const T f = F[n];
                const cx<T> s = useP ? v.p : v.q;
                re += f * s.x;
                im += f * s.y;
            }
            vr[c] = re;
            vi[c] = conj ? -im : im;
        }
        vfwd_project<T, FLUX>(d, w, j, vr, vi, nch, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
    }
}

// ---------------------------------------------------------------------------
// RK4 stage arithmetic on 3*M complex (6*M doubles), written without
// contraction like IntegrationBuffer::setAffine / addScaled
// (PortableRuntime/src/WVRungeKutta.cpp:140-176).

// acc = acc + scale * inc ; stage = base + cs * inc   (both from the same k)
__global__ void k_accumulate_and_stage(double* __restrict__ acc, const double* __restrict__ inc, double scale,
                                       const double* __restrict__ base, double cs, double* __restrict__ stage, int first, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double k = inc[i];
        acc[i] = first ? k : __dadd_rn(acc[i], __dmul_rn(scale, k));
        if (stage) stage[i] = __dadd_rn(base[i], __dmul_rn(cs, k));
    }
}

// The step's end: out = base + scale * (acc + k), with the arithmetic of
// k_accumulate_and_stage at weight 1 followed by base + scale * acc, in one
// pass (the final weighted sum is consumed here and not stored).
__global__ void k_rk4_finish(const double* __restrict__ acc, const double* __restrict__ inc, const double* base, double scale,
                             double* out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double a = __dadd_rn(acc[i], __dmul_rn(1.0, inc[i]));
        out[i] = __dadd_rn(base[i], __dmul_rn(scale, a));
    }
}

}  // namespace dev
}  // namespace wvgpu

namespace wvgpu {
namespace dev {
// out = a*x + b*y (y may be null); n doubles
__global__ void k_lincomb(double* __restrict__ out, double a, const double* __restrict__ x, double b,
                          const double* __restrict__ y, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = y ? __fma_rn(a, x[i], __dmul_rn(b, y[i])) : __dmul_rn(a, x[i]);
}
// One stage of the RK4 backward sweep after a flux VJP s: the step's
// cotangent acc = x + s (first stage) or acc += s, and the next stage's flux
// cotangent kb = a x + b s, with k_lincomb's rounding.
__global__ void k_adj_stage(double* __restrict__ acc, bool first, double* __restrict__ kb, double a,
                            const double* __restrict__ x, double b, const double* __restrict__ s, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double xi = x[i], si = s[i];
        acc[i] = first ? __fma_rn(1.0, xi, __dmul_rn(1.0, si)) : __dadd_rn(acc[i], si);
        kb[i] = __fma_rn(a, xi, __dmul_rn(b, si));
    }
}
// out += x
__global__ void k_accumulate(double* __restrict__ out, const double* __restrict__ x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] += x[i];
}
// RK4 dense output: out = iw y0 + ew y1 + isw k1 + esw k4, summed left to right
// without contraction (WVFixedStepRK4::evaluateDenseOutput); grid.y = component.
__global__ void k_rk4_dense(const double* __restrict__ y0, const double* __restrict__ y1, const double* __restrict__ k1,
                            const double* __restrict__ k4, double iw, double ew, double isw, double esw, double* Ap,
                            double* Am, double* A0, size_t M2) {
    const int c = blockIdx.y;
    double* dst = c == 0 ? Ap : (c == 1 ? Am : A0);
    const size_t o = c * M2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < M2; i += (size_t)gridDim.x * blockDim.x) {
        double v = __dadd_rn(__dmul_rn(iw, y0[o + i]), __dmul_rn(ew, y1[o + i]));
        v = __dadd_rn(v, __dmul_rn(isw, k1[o + i]));
        dst[i] = __dadd_rn(v, __dmul_rn(esw, k4[o + i]));
    }
}
}  // namespace dev
}  // namespace wvgpu

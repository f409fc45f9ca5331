// Vertical transforms as FFTs of the even / odd extension over z (every
// precision), the way the reference computes them (FFTW REDFT00 /
// RODFT00, WVNativeFFTWEngine.cpp:154; exact definitions
// WVReferenceFFTEngine.cpp:88-107), instead of the dense folded contraction.
//
// With L = Nz - 1 and a line y[0 .. 2L-1] holding a cosine-family channel C_j
// and a sine-family channel D_j of the same retained column,
//   y[0] = C_0 / 2,  y[L] = C_L (when j = L is kept),
//   y[j] = (C_j + i D_j) / 2,  y[2L-j] = (C_j - i D_j) / 2   (1 <= j < L),
// the forward FFT F[n] = sum_k y[k] exp(-i pi k n / L) splits into a part even
// in n and a part odd in n:
//   (F[n] + F[2L-n]) / 2 = C_0 / 2 + sum_{j>=1} C_j cos(pi j n / L)   (Ccos)
//   (F[n] - F[2L-n]) / 2 = sum_{j>=1} D_j sin(pi j n / L)             (Csin)
// for n = 0 .. L (the odd part is zero at n = 0 and n = L).  One complex FFT
// of length 2L per pair of channels: per retained column the values pair
// (u, w) and (v, eta), the z-derivatives (m_j w, -m_j u) and (m_j eta, -m_j v)
// (kernel.cpp:246-267; CcosM = m Ccos, CsinM = -m Csin).  At 256x256x129 that
// is 4 FFTs of 256 points per column (~41 kflop) against ~177 kflop for the
// dense folded contraction.
//
// The forward transform (normalizeForwardDCT / DST, kernel.cpp:176-193) pairs
// a cosine-family z-grid channel c_z with a sine-family one s_z the same way:
// y[0] = c_0, y[L] = c_L, y[z] = c_z + s_z, y[2L-z] = c_z - s_z, and
//   X_cos[j] = (F[j] + F[2L-j]) / 2 / (L Nx Ny)   (halved at j = L)
//   X_sin[j] = i (F[j] - F[2L-j]) / 2 / (L Nx Ny)
// (Fcos, Fsin with their endpoint weights and the horizontal scale), then the
// projection of k_vfwd (vfwd_project) per (mode, j).
//
// The adjoints (k_vfwd_adj_fft, k_vinv_adj_fft) are the transposed maps on the
// same lines: the transposed forward matrices are an inverse-type line
// (y[0] = X_0, y[L] = X_L / 2, y[j] = (X_j + i Y_j) / 2 ...) scaled by
// w_z / (L Nx Ny) (w_z = 2 inside, 1 at the ends) or 2 / (L Nx Ny); the
// transposed inverse matrices a forward-type line (y[0] = o_0, y[L] = o_L,
// y[z] = (o_z + i s_z) / 2, y[2L-z] = (o_z - i s_z) / 2) with Ccos's 1/2 at
// j = 0 and +/- m_j for the z-derivative channels.
#pragma once

#include "wv_adjoint.cuh"
#include "wv_kernels.cuh"
#include "wv_warpfft.cuh"

namespace wvgpu {
namespace dev {

// FFT lines per CTA: 4 (256 threads, one radix-4 butterfly each at 2L = 256)
// in every precision.  8 lines per CTA in FP32 measured slower at 256x256x129
// and 512x512x257 (twice the shared memory, fewer CTAs per SM: 0.12 against
// 0.09 ms for the forward transform at 256, 1.58 against 1.04 ms for the
// inverse at 512) and only a few percent faster at 128x128x65.
template <typename T> struct VzLines { static constexpr int value = 4; };

template <typename T, bool FLUX>
struct VzShape {
    static constexpr int lines = FLUX ? 4 : 2;                   // lines per retained column
    static constexpr int modes = VzLines<T>::value / lines;     // retained columns per CTA
};

// Shared memory of k_vinv_fft: field spectra [4][Nj][modes], two line buffers
// [lines][2L] and the twiddles [2L].
template <typename T>
inline size_t smem_vinv_fft(int Nj, int N2, int modes) {
    return (static_cast<size_t>(4) * Nj * modes + 2 * static_cast<size_t>(VzLines<T>::value) * N2 + N2) * sizeof(cx<T>);
}

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256) k_vinv_fft(DescDev d, const double* __restrict__ Ap, const double* __restrict__ Am,
                                                 const double* __restrict__ A0, double elapsed, cx<T>* __restrict__ zspec,
                                                 unsigned long long* __restrict__ maxSpeedBits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kLines = VzShape<T, FLUX>::lines, kModes = VzShape<T, FLUX>::modes, kVzLines = VzLines<T>::value;
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, L = Nz - 1, N2 = d.fz.N;
    cx<T>* fld = reinterpret_cast<cx<T>*>(smem_raw);   // [4][Nj][kModes]
    cx<T>* bufA = fld + 4 * Nj * kModes;               // [kVzLines][N2]
    cx<T>* bufB = bufA + kVzLines * N2;
    cx<T>* tw = bufB + kVzLines * N2;                  // [N2]
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        zspec += (size_t)member * Nz * P;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && maxSpeedBits) maxSpeedBits[member] = 0ull;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < kVzLines * N2; i += blockDim.x) bufA[i] = mk<T>(T(0), T(0));
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it / Nj, j = it - mi * Nj;
        cx<T> f[4];
        vinv_field_spectra<T>(d, Ap, Am, A0, elapsed, m0 + mi, j, f);
#pragma unroll
        for (int q = 0; q < 4; ++q) fld[(q * Nj + j) * kModes + mi] = f[q];
    }
    __syncthreads();
    // lines: y[j] = (C_j + i D_j) / 2, y[2L-j] = (C_j - i D_j) / 2, y[0] = C_0 / 2, y[L] = C_L
    const T* mz = reinterpret_cast<const T*>(d.tMz);
    const T half = T(0.5f);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it / Nj, j = it - mi * Nj;
        const cx<T> U = fld[(0 * Nj + j) * kModes + mi], V = fld[(1 * Nj + j) * kModes + mi];
        const cx<T> W = fld[(2 * Nj + j) * kModes + mi], E = fld[(3 * Nj + j) * kModes + mi];
        cx<T> C[kLines], D[kLines];
        C[0] = U; D[0] = W;
        C[1] = V; D[1] = E;
        if constexpr (FLUX) {
            const T m = mz[j];
            C[2] = mk<T>(m * W.x, m * W.y); D[2] = mk<T>(-(m * U.x), -(m * U.y));
            C[3] = mk<T>(m * E.x, m * E.y); D[3] = mk<T>(-(m * V.x), -(m * V.y));
        }
#pragma unroll
        for (int l = 0; l < kLines; ++l) {
            cx<T>* y = bufA + (mi * kLines + l) * N2;
            if (j == 0) {
                y[0] = mk<T>(C[l].x * half, C[l].y * half);
            } else if (j == L) {
                y[L] = C[l];
            } else {
                // (C +/- i D) / 2
                const cx<T> c = mk<T>(C[l].x * half, C[l].y * half);
                const cx<T> id = mk<T>(-(D[l].y * half), D[l].x * half);
                y[j] = cadd<T>(c, id);
                y[N2 - j] = csub<T>(c, id);
            }
        }
    }
    __syncthreads();
    const cx<T>* F = fft_lines<T, false>(bufA, bufB, d.fz, kVzLines, N2, tw);
    // even part -> cosine channel, odd part -> sine channel, n = 0 .. L
    int derivChan[4] = {-1, -1, -1, -1};
    if constexpr (FLUX)
        for (int t = 0; t < d.nt; ++t) derivChan[d.tq[t]] = 4 + t;
    for (int it = threadIdx.x; it < nm * kLines * (L + 1); it += blockDim.x) {
        const int n = it % (L + 1);
        const int rest = it / (L + 1);
        const int l = rest % kLines, mi = rest / kLines;
        const cx<T>* row = F + (mi * kLines + l) * N2;
        const cx<T> a = row[n];
        cx<T> ev = a, od = mk<T>(T(0), T(0));
        if (n != 0 && n != L) {
            const cx<T> b = row[N2 - n];
            ev = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
            od = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
        }
        int chC, chS;  // channels of the cosine and sine parts
        if (l == 0) { chC = 0; chS = 2; }
        else if (l == 1) { chC = 1; chS = 3; }
        else if (l == 2) { chC = derivChan[2]; chS = derivChan[0]; }
        else { chC = derivChan[3]; chS = derivChan[1]; }
        const int mode = m0 + mi;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        if (chC >= 0) {
            cx<T>* base = zspec + (size_t)chC * d.zTotal * P + (size_t)n * P;
            base[pos] = ev;
            if (cpos >= 0) base[cpos] = cconj<T>(ev);
        }
        if (chS >= 0) {
            cx<T>* base = zspec + (size_t)chS * d.zTotal * P + (size_t)n * P;
            base[pos] = od;
            if (cpos >= 0) base[cpos] = cconj<T>(od);
        }
    }
}

// Shared memory of k_vfwd_fft: two line buffers [lines][2L] and the twiddles [2L].
template <typename T>
inline size_t smem_vfwd_fft(int N2) {
    return (2 * static_cast<size_t>(VzLines<T>::value) * N2 + N2) * sizeof(cx<T>);
}

// retained columns per CTA of k_vfwd_fft / k_vfwd_adj_fft: lines (u | w) and (v | eta) each
template <typename T>
__host__ __device__ constexpr int vf_modes() { return VzLines<T>::value / 2; }

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256) k_vfwd_fft(DescDev d, const cx<T>* __restrict__ fspec, int nch, double elapsed,
                                                 const double* __restrict__ Ap, const double* __restrict__ Am,
                                                 const double* __restrict__ A0, const unsigned long long* __restrict__ maxSpeedBits,
                                                 int applyDamping, double* __restrict__ Fp, double* __restrict__ Fm,
                                                 double* __restrict__ F0) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kVzLines = VzLines<T>::value, kVfModes = vf_modes<T>();
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, L = Nz - 1, N2 = d.fz.N;
    cx<T>* bufA = reinterpret_cast<cx<T>*>(smem_raw);  // [kVzLines][N2]
    cx<T>* bufB = bufA + kVzLines * N2;
    cx<T>* tw = bufB + kVzLines * N2;                 // [N2]
    const int m0 = blockIdx.x * kVfModes;
    const int nm = min(kVfModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        if (Ap) { Ap += o; Am += o; A0 += o; }
        Fp += o; Fm += o; F0 += o;
        fspec += (size_t)member * Nz * P;
        if (maxSpeedBits) maxSpeedBits += member;
    }
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < kVzLines * N2; i += blockDim.x) bufA[i] = mk<T>(T(0), T(0));
    // channel holding each field slot q (0 u, 1 v: cosine family; 2 w, 3 eta: sine family)
    int chanOfQ[4] = {-1, -1, -1, -1};
    for (int c = 0; c < nch; ++c) chanOfQ[FLUX ? d.tq[c] : ((d.hydrostatic && c == 2) ? 3 : c)] = c;
    __syncthreads();
    for (int it = threadIdx.x; it < nm * 2 * (L + 1); it += blockDim.x) {
        const int z = it % (L + 1);
        const int rest = it / (L + 1);
        const int l = rest & 1, mi = rest >> 1;
        const int pos = d.modePos[m0 + mi];
        const int cc = l == 0 ? chanOfQ[0] : chanOfQ[1], cs = l == 0 ? chanOfQ[2] : chanOfQ[3];
        const cx<T> cv = cc >= 0 ? fspec[(size_t)cc * d.zTotal * P + (size_t)z * P + pos] : mk<T>(T(0), T(0));
        cx<T>* y = bufA + (mi * 2 + l) * N2;
        if (z == 0 || z == L) {
            y[z] = cv;
        } else {
            const cx<T> sv = cs >= 0 ? fspec[(size_t)cs * d.zTotal * P + (size_t)z * P + pos] : mk<T>(T(0), T(0));
            y[z] = cadd<T>(cv, sv);
            y[N2 - z] = csub<T>(cv, sv);
        }
    }
    __syncthreads();
    const cx<T>* F = fft_lines<T, false>(bufA, bufB, d.fz, kVzLines, N2, tw);
    double maxSpeed = 0.0;
    if (FLUX && applyDamping) maxSpeed = __longlong_as_double((long long)*maxSpeedBits);
    const T sc = T(1.0 / (static_cast<double>(L) * static_cast<double>(d.Nx) * static_cast<double>(d.Ny)));
    const T half = T(0.5f);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it % nm, j = it / nm;
        const int mode = m0 + mi;
        const int w = d.modeWV[mode];
        const bool conj = d.modeFlags[mode] & 1;
        // transformed slots (canonical frame): 0 u, 1 v (cosine), 2 w, 3 eta (sine)
        cx<T> X[4];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const cx<T>* row = F + (mi * 2 + l) * N2;
            const cx<T> a = row[j];
            cx<T> ev = a, od = mk<T>(T(0), T(0));
            if (j != 0 && j != L) {
                const cx<T> b = row[N2 - j];
                ev = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
                od = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
            }
            const T scC = j == L ? sc * half : sc;
            X[l] = mk<T>(ev.x * scC, ev.y * scC);
            X[2 + l] = mk<T>(-(od.y * sc), od.x * sc);  // i * odd part
        }
        T vr[4] = {T(0), T(0), T(0), T(0)}, vi[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            const int q = FLUX ? d.tq[c] : ((d.hydrostatic && c == 2) ? 3 : c);
            const cx<T> v = q == 0 ? X[0] : q == 1 ? X[1] : q == 2 ? X[2] : X[3];
            vr[c] = v.x;
            vi[c] = conj ? -v.y : v.y;
        }
        vfwd_project<T, FLUX>(d, w, j, vr, vi, nch, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
    }
}

// ---------------------------------------------------------------------------
// The flux's vertical transforms on register-resident warp lines (mixed and
// FP32X2 handles, 2L = 32 R points): one line per warp, built in registers
// from the same entries as k_vinv_fft / k_vfwd_fft, transformed by fft_P (no
// block barrier inside the FFT; paired FP32 in split form), then parked in a
// per-warp line buffer for the even / odd split.  Line buffers are padded by
// one value every 8 so that the lane-bit-reversed stores of fft_P's output
// meet no bank conflicts.

constexpr int kVwWarps = 8;  // lines per CTA (256 threads)
__host__ __device__ inline int vw_pad(int i) { return i + (i >> 3); }
__host__ __device__ inline int vw_line_len(int N2) { return N2 + N2 / 8; }

// k_vinv_wfft: field spectra [4][Nj][2 modes], twiddles [2L], line buffers [8][2L + 2L/8]
template <typename T>
inline size_t smem_vinv_wfft(int Nj, int N2) {
    return (static_cast<size_t>(4) * Nj * (kVwWarps / 4) + N2 + static_cast<size_t>(kVwWarps) * vw_line_len(N2)) *
           sizeof(cx<T>);
}
// k_vfwd_wfft: twiddles [2L], line buffers [8][2L + 2L/8]
template <typename T>
inline size_t smem_vfwd_wfft(int N2) {
    return (N2 + static_cast<size_t>(kVwWarps) * vw_line_len(N2)) * sizeof(cx<T>);
}

// fft_P output (register k1 of lane t = F[k1 + R brev5(t)]) into a padded line buffer
template <typename T, int R>
__device__ __forceinline__ void vw_park(cx<T>* F, const cx<T> (&v)[R], int lane) {
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) F[vw_pad(p_index<R>(k1, lane))] = v[k1];
    __syncwarp();
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_vinv_wfft(DescDev d, const double* __restrict__ Ap, const double* __restrict__ Am,
                                                  const double* __restrict__ A0, double elapsed, cx<T>* __restrict__ zspec,
                                                  unsigned long long* __restrict__ maxSpeedBits) {
    constexpr int N2 = 32 * R, kModes = kVwWarps / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, L = Nz - 1;
    cx<T>* fld = reinterpret_cast<cx<T>*>(smem_raw);  // [4][Nj][kModes]
    cx<T>* tw = fld + 4 * Nj * kModes;                // [N2]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cx<T>* F = tw + N2 + warp * vw_line_len(N2);
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        zspec += (size_t)member * Nz * P;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && maxSpeedBits) maxSpeedBits[member] = 0ull;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it / Nj, j = it - mi * Nj;
        cx<T> f[4];
        vinv_field_spectra<T>(d, Ap, Am, A0, elapsed, m0 + mi, j, f);
#pragma unroll
        for (int q = 0; q < 4; ++q) fld[(q * Nj + j) * kModes + mi] = f[q];
    }
    __syncthreads();
    const int mi = warp >> 2, l = warp & 3;  // mode, line: (u | w), (v | eta), (m w | -m u), (m eta | -m v)
    if (mi >= nm) return;
    const T* mz = reinterpret_cast<const T*>(d.tMz);
    const T half = T(0.5f);
    // line entries y[k], k = lane + 32 r: y[0] = C_0 / 2, y[L] = C_L,
    // y[j] = (C_j + i D_j) / 2, y[2L-j] = (C_j - i D_j) / 2
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int k = lane + 32 * r;
        const int j = k <= L ? k : N2 - k;
        cx<T> val = mk<T>(T(0), T(0));
        if (j < Nj) {
            const cx<T> U = fld[(0 * Nj + j) * kModes + mi], V = fld[(1 * Nj + j) * kModes + mi];
            const cx<T> W = fld[(2 * Nj + j) * kModes + mi], E = fld[(3 * Nj + j) * kModes + mi];
            cx<T> C, D;
            if (l == 0) { C = U; D = W; }
            else if (l == 1) { C = V; D = E; }
            else {
                const T m = mz[j];
                if (l == 2) { C = mk<T>(m * W.x, m * W.y); D = mk<T>(-(m * U.x), -(m * U.y)); }
                else { C = mk<T>(m * E.x, m * E.y); D = mk<T>(-(m * V.x), -(m * V.y)); }
            }
            if (k == 0) {
                val = mk<T>(C.x * half, C.y * half);
            } else if (k == L) {
                val = C;
            } else {
                const cx<T> c = mk<T>(C.x * half, C.y * half);
                const cx<T> id = mk<T>(-(D.y * half), D.x * half);
                val = k < L ? cadd<T>(c, id) : csub<T>(c, id);
            }
        }
        v[r] = val;
    }
    fft_P<T, R, false>(v, tw, lane);
    vw_park<T, R>(F, v, lane);
    // even part -> cosine channel, odd part -> sine channel, n = 0 .. L
    int derivChan[4] = {-1, -1, -1, -1};
    for (int t = 0; t < d.nt; ++t) derivChan[d.tq[t]] = 4 + t;
    int chC, chS;
    if (l == 0) { chC = 0; chS = 2; }
    else if (l == 1) { chC = 1; chS = 3; }
    else if (l == 2) { chC = derivChan[2]; chS = derivChan[0]; }
    else { chC = derivChan[3]; chS = derivChan[1]; }
    const int mode = m0 + mi;
    const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
    for (int n = lane; n <= L; n += 32) {
        const cx<T> a = F[vw_pad(n)];
        cx<T> ev = a, od = mk<T>(T(0), T(0));
        if (n != 0 && n != L) {
            const cx<T> b = F[vw_pad(N2 - n)];
            ev = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
            od = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
        }
        if (chC >= 0) {
            cx<T>* base = zspec + (size_t)chC * d.zTotal * P + (size_t)n * P;
            base[pos] = ev;
            if (cpos >= 0) base[cpos] = cconj<T>(ev);
        }
        if (chS >= 0) {
            cx<T>* base = zspec + (size_t)chS * d.zTotal * P + (size_t)n * P;
            base[pos] = od;
            if (cpos >= 0) base[cpos] = cconj<T>(od);
        }
    }
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_vfwd_wfft(DescDev d, const cx<T>* __restrict__ fspec, int nch, double elapsed,
                                                  const double* __restrict__ Ap, const double* __restrict__ Am,
                                                  const double* __restrict__ A0, const unsigned long long* __restrict__ maxSpeedBits,
                                                  int applyDamping, double* __restrict__ Fp, double* __restrict__ Fm,
                                                  double* __restrict__ F0) {
    constexpr int N2 = 32 * R, kModes = kVwWarps / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, L = Nz - 1;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);  // [N2]
    cx<T>* lines = tw + N2;                           // [8][N2 + N2/8]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        if (Ap) { Ap += o; Am += o; A0 += o; }
        Fp += o; Fm += o; F0 += o;
        fspec += (size_t)member * Nz * P;
        if (maxSpeedBits) maxSpeedBits += member;
    }
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    // channel holding each field slot q (0 u, 1 v: cosine family; 2 w, 3 eta: sine family)
    int chanOfQ[4] = {-1, -1, -1, -1};
    for (int c = 0; c < nch; ++c) chanOfQ[d.tq[c]] = c;
    __syncthreads();
    const int mi = warp >> 1, l = warp & 1;  // mode, line: (u | w), (v | eta)
    if (mi < nm) {
        const int pos = d.modePos[m0 + mi];
        const int cc = l == 0 ? chanOfQ[0] : chanOfQ[1], cs = l == 0 ? chanOfQ[2] : chanOfQ[3];
        auto at = [&](int ch, int z) {
            return ch >= 0 ? fspec[(size_t)ch * d.zTotal * P + (size_t)z * P + pos] : mk<T>(T(0), T(0));
        };
        // y[0] = c_0, y[L] = c_L, y[z] = c_z + s_z, y[2L-z] = c_z - s_z
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int k = lane + 32 * r;
            const int z = k <= L ? k : N2 - k;
            const cx<T> cv = at(cc, z);
            v[r] = (k == 0 || k == L) ? cv : (k < L ? cadd<T>(cv, at(cs, z)) : csub<T>(cv, at(cs, z)));
        }
        fft_P<T, R, false>(v, tw, lane);
        vw_park<T, R>(lines + warp * vw_line_len(N2), v, lane);
    }
    __syncthreads();  // both lines of every mode parked
    double maxSpeed = 0.0;
    if (applyDamping) maxSpeed = __longlong_as_double((long long)*maxSpeedBits);
    const T sc = T(1.0 / (static_cast<double>(L) * static_cast<double>(d.Nx) * static_cast<double>(d.Ny)));
    const T half = T(0.5f);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int m = it % nm, j = it / nm;
        const int mode = m0 + m;
        const int w = d.modeWV[mode];
        const bool conj = d.modeFlags[mode] & 1;
        cx<T> X[4];
#pragma unroll
        for (int ll = 0; ll < 2; ++ll) {
            const cx<T>* row = lines + (m * 2 + ll) * vw_line_len(N2);
            const cx<T> a = row[vw_pad(j)];
            cx<T> ev = a, od = mk<T>(T(0), T(0));
            if (j != 0 && j != L) {
                const cx<T> b = row[vw_pad(N2 - j)];
                ev = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
                od = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
            }
            const T scC = j == L ? sc * half : sc;
            X[ll] = mk<T>(ev.x * scC, ev.y * scC);
            X[2 + ll] = mk<T>(-(od.y * sc), od.x * sc);  // i * odd part
        }
        T vr[4] = {T(0), T(0), T(0), T(0)}, vi[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (c >= nch) break;
            const int q = d.tq[c];
            const cx<T> v = q == 0 ? X[0] : q == 1 ? X[1] : q == 2 ? X[2] : X[3];
            vr[c] = v.x;
            vi[c] = conj ? -v.y : v.y;
        }
        vfwd_project<T, true>(d, w, j, vr, vi, nch, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
    }
}

// The flux VJP's vertical maps on warp-register lines (mixed and FP32X2,
// 2L = 32 R): the lines of k_vfwd_adj_fft / k_vinv_adj_fft, one per warp.

// k_vfwd_adj_wfft: cotangent targets [4][Nj][4 modes], twiddles, line buffers
template <typename T>
inline size_t smem_vfwd_adj_wfft(int Nj, int N2) {
    return (static_cast<size_t>(4) * Nj * (kVwWarps / 2) + N2 + static_cast<size_t>(kVwWarps) * vw_line_len(N2)) *
           sizeof(cx<T>);
}
// k_vinv_adj_wfft: twiddles, line buffers
template <typename T>
inline size_t smem_vinv_adj_wfft(int N2) {
    return (N2 + static_cast<size_t>(kVwWarps) * vw_line_len(N2)) * sizeof(cx<T>);
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_vfwd_adj_wfft(DescDev d, const double* __restrict__ Fpb, const double* __restrict__ Fmb,
                                                      const double* __restrict__ F0b, double elapsed, cx<T>* __restrict__ zadj) {
    constexpr int N2 = 32 * R, kModes = kVwWarps / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, nt = d.nt, L = Nz - 1;
    cx<T>* tv = reinterpret_cast<cx<T>*>(smem_raw);  // [4][Nj][kModes]: target cotangents per slot q
    cx<T>* tw = tv + 4 * Nj * kModes;                // [N2]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    cx<T>* F = tw + N2 + warp * vw_line_len(N2);
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    int tOfQ[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) tOfQ[d.tq[t]] = t;
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it % nm, j = it / nm;
        cx<T> vt[4];
        vfwd_adj_values<T>(d, Fpb, Fmb, F0b, elapsed, d.modeWV[m0 + mi], j, vt);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int t = tOfQ[q];
            tv[(q * Nj + j) * kModes + mi] = t < 0 ? mk<T>(T(0), T(0)) : (t == 0 ? vt[0] : t == 1 ? vt[1] : t == 2 ? vt[2] : vt[3]);
        }
    }
    __syncthreads();
    const int mi = warp >> 1, l = warp & 1;  // mode, line: (u | w), (v | eta)
    if (mi >= nm) return;
    const T half = T(0.5f);
    // y[0] = X_0, y[L] = X_L / 2, y[j] = (X_j + i Y_j) / 2, y[2L-j] = (X_j - i Y_j) / 2
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int k = lane + 32 * r;
        const int j = k <= L ? k : N2 - k;
        cx<T> val = mk<T>(T(0), T(0));
        if (j < Nj) {
            const cx<T> C = tv[(l * Nj + j) * kModes + mi], D = tv[((2 + l) * Nj + j) * kModes + mi];
            if (k == 0) {
                val = C;
            } else if (k == L) {
                val = mk<T>(C.x * half, C.y * half);
            } else {
                const cx<T> c = mk<T>(C.x * half, C.y * half);
                const cx<T> id = mk<T>(-(D.y * half), D.x * half);
                val = k < L ? cadd<T>(c, id) : csub<T>(c, id);
            }
        }
        v[r] = val;
    }
    fft_P<T, R, false>(v, tw, lane);
    vw_park<T, R>(F, v, lane);
    const T sc = T(1.0 / (static_cast<double>(L) * static_cast<double>(d.Nx) * static_cast<double>(d.Ny)));
    const T sc2 = sc + sc;
    const int mode = m0 + mi;
    const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
    const bool conj = d.modeFlags[mode] & 1;
    const int tc = l == 0 ? tOfQ[0] : tOfQ[1], ts = l == 0 ? tOfQ[2] : tOfQ[3];
    for (int z = lane; z <= L; z += 32) {
        const cx<T> a = F[vw_pad(z)];
        cx<T> vc, vs;
        if (z == 0 || z == L) {
            vc = mk<T>(a.x * sc, a.y * sc);
            vs = mk<T>(T(0), T(0));
        } else {
            const cx<T> b = F[vw_pad(N2 - z)];
            vc = mk<T>((a.x + b.x) * sc, (a.y + b.y) * sc);  // w_z (F[z] + F[2L-z]) / 2 with w_z = 2
            vs = mk<T>((a.x - b.x) * half * sc2, (a.y - b.y) * half * sc2);
        }
        if (tc >= 0) {
            cx<T>* base = zadj + (size_t)tc * Nz * P + (size_t)z * P;
            base[pos] = conj ? cconj<T>(vc) : vc;
            if (cpos >= 0) base[cpos] = mk<T>(T(0), T(0));
        }
        if (ts >= 0) {
            cx<T>* base = zadj + (size_t)ts * Nz * P + (size_t)z * P;
            base[pos] = conj ? cconj<T>(vs) : vs;
            if (cpos >= 0) base[cpos] = mk<T>(T(0), T(0));
        }
    }
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_vinv_adj_wfft(DescDev d, const cx<T>* __restrict__ fadj, double elapsed,
                                                      double* __restrict__ Apb, double* __restrict__ Amb,
                                                      double* __restrict__ A0b) {
    constexpr int N2 = 32 * R, kModes = kVwWarps / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, nt = d.nt, L = Nz - 1;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);  // [N2]
    cx<T>* lines = tw + N2;                           // [8][N2 + N2/8]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    int derivChan[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) derivChan[d.tq[t]] = 4 + t;
    const T half = T(0.5f);
    __syncthreads();
    const int mi = warp >> 2, l = warp & 3;
    if (mi < nm) {
        const int mode = m0 + mi;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const unsigned char flags = d.modeFlags[mode];
        int chC, chS;
        if (l == 0) { chC = 0; chS = 2; }
        else if (l == 1) { chC = 1; chS = 3; }
        else if (l == 2) { chC = derivChan[2]; chS = derivChan[0]; }
        else { chC = derivChan[3]; chS = derivChan[1]; }
        // stored row + conjugated completion row, frame of k_vinv (as k_vinv_adj's gather)
        auto colval = [&](int ch, int z) -> cx<T> {
            if (ch < 0) return mk<T>(T(0), T(0));
            const cx<T>* r = fadj + ((size_t)ch * Nz + z) * P;
            cx<T> v = r[pos];
            if (cpos >= 0) { const cx<T> c = r[cpos]; v = mk<T>(v.x + c.x, v.y - c.y); }
            if (flags & 2) v.y = T(0);
            if (flags & 1) v.y = -v.y;
            return v;
        };
        // y[0] = o_0, y[L] = o_L, y[z] = (o_z + i s_z) / 2, y[2L-z] = (o_z - i s_z) / 2
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int k = lane + 32 * r;
            const int z = k <= L ? k : N2 - k;
            const cx<T> o = colval(chC, z);
            if (k == 0 || k == L) {
                v[r] = o;
            } else {
                const cx<T> sv = colval(chS, z);
                const cx<T> c = mk<T>(o.x * half, o.y * half);
                const cx<T> id = mk<T>(-(sv.y * half), sv.x * half);
                v[r] = k < L ? cadd<T>(c, id) : csub<T>(c, id);
            }
        }
        fft_P<T, R, false>(v, tw, lane);
        vw_park<T, R>(lines + warp * vw_line_len(N2), v, lane);
    }
    __syncthreads();  // the four lines of every mode parked
    const T* mz = reinterpret_cast<const T*>(d.tMz);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int m = it % nm, j = it / nm;
        const int w = d.modeWV[m0 + m];
        cx<T> Ev[4], Od[4];
#pragma unroll
        for (int ll = 0; ll < 4; ++ll) {
            const cx<T>* row = lines + (m * 4 + ll) * vw_line_len(N2);
            const cx<T> a = row[vw_pad(j)];
            if (j == 0 || j == L) {
                Ev[ll] = j == 0 ? mk<T>(a.x * half, a.y * half) : a;  // Ccos's 1/2 at j = 0
                Od[ll] = mk<T>(T(0), T(0));
            } else {
                const cx<T> b = row[vw_pad(N2 - j)];
                Ev[ll] = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
                Od[ll] = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
            }
        }
        const T mj = mz[j];
        const cx<T> ubT = mk<T>(Ev[0].x - mj * Od[2].x, Ev[0].y - mj * Od[2].y);
        const cx<T> wbT = mk<T>(Od[0].x + mj * Ev[2].x, Od[0].y + mj * Ev[2].y);
        const cx<T> vbT = mk<T>(Ev[1].x - mj * Od[3].x, Ev[1].y - mj * Od[3].y);
        const cx<T> nbT = mk<T>(Od[1].x + mj * Ev[3].x, Od[1].y + mj * Ev[3].y);
        vinv_adj_store<T>(d, j + Nj * w, elapsed, ubT, vbT, wbT, nbT, Apb, Amb, A0b);
    }
}

// Shared memory of the adjoint kernels: two line buffers and the twiddles.
template <typename T>
inline size_t smem_vadj_fft(int N2) {
    return (2 * static_cast<size_t>(VzLines<T>::value) * N2 + N2) * sizeof(cx<T>);
}

// Transpose of the projection + forward vertical transform (k_vfwd_adj) with the
// transposed forward matrices as FFTs: per retained column the target pairs
// (u | w) and (v | eta).  Single-state handles, like k_vfwd_adj.
template <typename T>
__global__ void __launch_bounds__(256) k_vfwd_adj_fft(DescDev d, const double* __restrict__ Fpb, const double* __restrict__ Fmb,
                                                     const double* __restrict__ F0b, double elapsed, cx<T>* __restrict__ zadj) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kVzLines = VzLines<T>::value, kVfModes = vf_modes<T>();
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, nt = d.nt, L = Nz - 1, N2 = d.fz.N;
    cx<T>* bufA = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* bufB = bufA + kVzLines * N2;
    cx<T>* tw = bufB + kVzLines * N2;
    const int m0 = blockIdx.x * kVfModes;
    const int nm = min(kVfModes, d.Nkl - m0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < kVzLines * N2; i += blockDim.x) bufA[i] = mk<T>(T(0), T(0));
    int tOfQ[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) tOfQ[d.tq[t]] = t;
    __syncthreads();
    const T half = T(0.5f);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it % nm, j = it / nm;
        cx<T> vt[4];
        vfwd_adj_values<T>(d, Fpb, Fmb, F0b, elapsed, d.modeWV[m0 + mi], j, vt);
        cx<T> X[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int t = tOfQ[q];
            X[q] = t < 0 ? mk<T>(T(0), T(0)) : (t == 0 ? vt[0] : t == 1 ? vt[1] : t == 2 ? vt[2] : vt[3]);
        }
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const cx<T> C = X[l], D = X[2 + l];  // cosine target, sine target
            cx<T>* y = bufA + (mi * 2 + l) * N2;
            if (j == 0) {
                y[0] = C;
            } else if (j == L) {
                y[L] = mk<T>(C.x * half, C.y * half);
            } else {
                const cx<T> c = mk<T>(C.x * half, C.y * half);
                const cx<T> id = mk<T>(-(D.y * half), D.x * half);
                y[j] = cadd<T>(c, id);
                y[N2 - j] = csub<T>(c, id);
            }
        }
    }
    __syncthreads();
    const cx<T>* F = fft_lines<T, false>(bufA, bufB, d.fz, kVzLines, N2, tw);
    const T sc = T(1.0 / (static_cast<double>(L) * static_cast<double>(d.Nx) * static_cast<double>(d.Ny)));
    const T sc2 = sc + sc;
    for (int it = threadIdx.x; it < nm * 2 * (L + 1); it += blockDim.x) {
        const int z = it % (L + 1);
        const int rest = it / (L + 1);
        const int l = rest & 1, mi = rest >> 1;
        const int mode = m0 + mi;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const bool conj = d.modeFlags[mode] & 1;
        const cx<T>* row = F + (mi * 2 + l) * N2;
        const cx<T> a = row[z];
        cx<T> vc, vs;
        if (z == 0 || z == L) {
            vc = mk<T>(a.x * sc, a.y * sc);
            vs = mk<T>(T(0), T(0));
        } else {
            const cx<T> b = row[N2 - z];
            vc = mk<T>((a.x + b.x) * sc, (a.y + b.y) * sc);  // w_z (F[z] + F[2L-z]) / 2 with w_z = 2
            vs = mk<T>((a.x - b.x) * half * sc2, (a.y - b.y) * half * sc2);
        }
        const int tc = l == 0 ? tOfQ[0] : tOfQ[1], ts = l == 0 ? tOfQ[2] : tOfQ[3];
        if (tc >= 0) {
            cx<T>* base = zadj + (size_t)tc * Nz * P + (size_t)z * P;
            base[pos] = conj ? cconj<T>(vc) : vc;
            if (cpos >= 0) base[cpos] = mk<T>(T(0), T(0));
        }
        if (ts >= 0) {
            cx<T>* base = zadj + (size_t)ts * Nz * P + (size_t)z * P;
            base[pos] = conj ? cconj<T>(vs) : vs;
            if (cpos >= 0) base[cpos] = mk<T>(T(0), T(0));
        }
    }
}

// Transpose of the flux's vertical inverse (k_vinv_adj<T, true>) with the
// transposed inverse matrices as FFTs: per retained column the channel pairs
// (U | W), (V | N) and the z-derivative channels (w_z | u_z), (eta_z | v_z),
// then the transposed assembly and phase (vinv_adj_store).  Single-state
// handles, like k_vinv_adj.
template <typename T>
__global__ void __launch_bounds__(256) k_vinv_adj_fft(DescDev d, const cx<T>* __restrict__ fadj, double elapsed,
                                                     double* __restrict__ Apb, double* __restrict__ Amb,
                                                     double* __restrict__ A0b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kVzLines = VzLines<T>::value, kLines = 4, kModes = kVzLines / kLines;
    const int Nj = d.Nj, Nz = d.Nz, P = d.positions, nt = d.nt, L = Nz - 1, N2 = d.fz.N;
    cx<T>* bufA = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* bufB = bufA + kVzLines * N2;
    cx<T>* tw = bufB + kVzLines * N2;
    const int m0 = blockIdx.x * kModes;
    const int nm = min(kModes, d.Nkl - m0);
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twz);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) tw[i] = twg[i];
    int derivChan[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) derivChan[d.tq[t]] = 4 + t;
    const T half = T(0.5f);
    // lines: y[0] = o_0, y[L] = o_L, y[z] = (o_z + i s_z) / 2, y[2L-z] = (o_z - i s_z) / 2
    for (int it = threadIdx.x; it < nm * kLines * (L + 1); it += blockDim.x) {
        const int z = it % (L + 1);
        const int rest = it / (L + 1);
        const int l = rest % kLines, mi = rest / kLines;
        const int mode = m0 + mi;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const unsigned char flags = d.modeFlags[mode];
        int chC, chS;
        if (l == 0) { chC = 0; chS = 2; }
        else if (l == 1) { chC = 1; chS = 3; }
        else if (l == 2) { chC = derivChan[2]; chS = derivChan[0]; }
        else { chC = derivChan[3]; chS = derivChan[1]; }
        // stored row + conjugated completion row, frame of k_vinv (as k_vinv_adj's gather)
        auto colval = [&](int ch) -> cx<T> {
            if (ch < 0) return mk<T>(T(0), T(0));
            const cx<T>* r = fadj + ((size_t)ch * Nz + z) * P;
            cx<T> v = r[pos];
            if (cpos >= 0) { const cx<T> c = r[cpos]; v = mk<T>(v.x + c.x, v.y - c.y); }
            if (flags & 2) v.y = T(0);
            if (flags & 1) v.y = -v.y;
            return v;
        };
        cx<T>* y = bufA + (mi * kLines + l) * N2;
        const cx<T> o = colval(chC);
        if (z == 0 || z == L) {
            y[z] = o;
        } else {
            const cx<T> sv = colval(chS);
            const cx<T> c = mk<T>(o.x * half, o.y * half);
            const cx<T> id = mk<T>(-(sv.y * half), sv.x * half);
            y[z] = cadd<T>(c, id);
            y[N2 - z] = csub<T>(c, id);
        }
    }
    __syncthreads();
    const cx<T>* F = fft_lines<T, false>(bufA, bufB, d.fz, kVzLines, N2, tw);
    const T* mz = reinterpret_cast<const T*>(d.tMz);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mi = it % nm, j = it / nm;
        const int w = d.modeWV[m0 + mi];
        cx<T> Ev[kLines], Od[kLines];
#pragma unroll
        for (int l = 0; l < kLines; ++l) {
            const cx<T>* row = F + (mi * kLines + l) * N2;
            const cx<T> a = row[j];
            if (j == 0 || j == L) {
                Ev[l] = j == 0 ? mk<T>(a.x * half, a.y * half) : a;  // Ccos's 1/2 at j = 0
                Od[l] = mk<T>(T(0), T(0));
            } else {
                const cx<T> b = row[N2 - j];
                Ev[l] = mk<T>((a.x + b.x) * half, (a.y + b.y) * half);
                Od[l] = mk<T>((a.x - b.x) * half, (a.y - b.y) * half);
            }
        }
        const T m = mz[j];
        // u_bar = Ccos^T U + (-m) Csin^T u_z;  w_bar = Csin^T W + m Ccos^T w_z; likewise v, eta
        const cx<T> ubT = mk<T>(Ev[0].x - m * Od[2].x, Ev[0].y - m * Od[2].y);
        const cx<T> wbT = mk<T>(Od[0].x + m * Ev[2].x, Od[0].y + m * Ev[2].y);
        const cx<T> vbT = mk<T>(Ev[1].x - m * Od[3].x, Ev[1].y - m * Od[3].y);
        const cx<T> nbT = mk<T>(Od[1].x + m * Ev[3].x, Od[1].y + m * Ev[3].y);
        vinv_adj_store<T>(d, j + Nj * w, elapsed, ubT, vbT, wbT, nbT, Apb, Amb, A0b);
    }
}

}  // namespace dev
}  // namespace wvgpu

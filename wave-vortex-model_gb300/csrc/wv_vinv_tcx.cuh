// Vertical inverse transform of the paired-FP32 (FP32X2) flux on the tensor
// cores: the same result as k_vinv<ff, true> (phase kernel.cpp:1186-1191, field
// spectra kernel.cpp:218-291 and WVCoefficientFormulas.hpp:23-58, Hermitian
// completion kernel.cpp:433-438, folded vertical inverse DCT-I / DST-I
// kernel.cpp:161-174, z-derivatives of the flux targets) with the
// dense contraction done as BF16 GEMMs of exact integer digit slices (the
// error-free splitting of Ozaki, Ogita, Oishi and Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012)).
//
// Every row of the A operand (mode, field, re|im over j) and every row of a
// matrix (output z over j) is scaled by a power of two so that its largest
// entry is below 1, and rounded to a 48-bit fixed-point integer written as six
// balanced base-256 digits, digit s in [-128, 128] stored as the BF16 value
// digit x 2^(-7-8s) (exact: at most 8 significant bits).  A digit product is
// an exact multiple of 2^(-14-8(s+t)) of magnitude <= 2^(-8(s+t)), so FP32
// sums of up to 2^10 / (level + 1) of a level's products stay exact.  Per
// accumulator (the even or odd half of j, <= 64 terms):
//   levels 0, 1 and 2 (s + t = 0, 1, 2) go to their own tensor-memory
//   accumulators and are exact; levels 3..5 (15 products) share a fourth one,
//   whose FP32 rounding is ~2^-48 of the row scale; levels >= 6 are dropped
//   (~2^-45).
// The z-derivative contractions take m_j on the A side (rows S_j m_j against
// Ccos and -Csin instead of S_j against m_j Ccos and -m_j Csin): the error of
// the scheme is relative to max_j |a_j| max_j |b_j| of a row pair, and the
// spectra fall with j while m_j grows.  The drain adds the four accumulators
// with error-free two-sums, scales by the two row exponents and stores paired
// FP32: ~1e-13 relative L2 error per contraction on 0.1 m/s spectrum states
// at 256x256x129 (the FP32X2 CUDA-core contraction is of the same order).
//
// One CTA (16 warps) takes 32 retained columns.  Pass 1 computes the paired
// FP32 field spectra of every (mode, j) once (FP64 phase, as k_vinv<ff>), keeps
// them in a per-CTA scratch row of global memory (L2) and reduces the row
// maxima of S and S m in shared memory.  Then per tile (0: u, v; 1: w, eta)
// and matrix half (values, then z-derivatives) the CTA writes the six digit
// slices of its 128 rows into shared memory, and per output pass (N rows of
// z, N <= 64) and j parity streams the pre-split matrix block by one bulk copy
// and issues the 21 digit products (tcgen05.mma kind::f16, M = 128, K = 16 per
// instruction) into four accumulators per parity (8 N <= 512 columns).  The
// drain folds out[n] = E + O, out[Nz-1-n] = E -/+ O as in k_vinv_tc.
#pragma once

#include "wv_kernels.cuh"
#include "wv_tc.cuh"
#include "wv_vinv_tc.cuh"

namespace wvgpu {
namespace dev {

constexpr int kTcxDigits = 6;        // digit slices per operand
constexpr uint32_t kTcxCols = 512;   // tensor-memory columns: 2 parities x 4 accumulators x N <= 64
constexpr int kTcxMaxBlocks = 64;    // matrix blocks per CTA (2 tiles x 2 halves x 2 parities x passes <= 8)

// Smallest E with |x| < 2^E for the largest |x| of a row (its FP32 bits);
// 0 for an all-zero row.
__device__ __forceinline__ int tcx_row_exponent(unsigned maxBits) {
    if (maxBits == 0u) return 0;
    const int be = static_cast<int>((maxBits >> 23) & 0xFFu);
    return be == 0 ? -126 : be - 126;
}

// x 2^e for e in [-252, 254] by two exact multiplications by powers of two.
__device__ __forceinline__ float tcx_scale(float x, int e) {
    const int h = e / 2;
    return __fmul_rn(__fmul_rn(x, __int_as_float((h + 127) << 23)), __int_as_float((e - h + 127) << 23));
}

// The six digit slices of v 2^-E as BF16 bits: Y = round(v 2^(47-E)) as an
// integer (|Y| <= 2^47), balanced base-256 digits from the bottom.
__device__ __forceinline__ void tcx_digits(ff v, int E, unsigned short (&out)[kTcxDigits]) {
    long long Y = __float2ll_rn(tcx_scale(v.hi, 47 - E)) + __float2ll_rn(tcx_scale(v.lo, 47 - E));
    int D[kTcxDigits];
#pragma unroll
    for (int s = kTcxDigits - 1; s >= 1; --s) {
        int dd = static_cast<int>(Y & 0xFFll);
        dd -= (dd & 0x80) << 1;  // [-128, 127]
        D[s] = dd;
        Y = (Y - dd) / 256;      // exact
    }
    D[0] = static_cast<int>(Y);  // [-128, 128]
#pragma unroll
    for (int s = 0; s < kTcxDigits; ++s) {
        const float f = __int2float_rn(D[s]) * __int_as_float((127 - 7 - 8 * s) << 23);  // exact
        out[s] = static_cast<unsigned short>(__float_as_uint(f) >> 16);
    }
}

// 2^e (a0 + a1 + a2 + a3) as a pair (error-free two-sums of the high words).
__device__ __forceinline__ ff tcx_combine(float a0, float a1, float a2, float a3, int e) {
    ff s = ff(a0) + ff(a1);
    s = s + ff(a2);
    s = s + ff(a3);
    return ff(tcx_scale(s.hi, e), tcx_scale(s.lo, e));
}


__global__ void __launch_bounds__(kTcThreads, 1)
k_vinv_tcx(DescDev d, const double* __restrict__ Ap, const double* __restrict__ Am, const double* __restrict__ A0,
           double elapsed, ff2* __restrict__ zspec, unsigned long long* __restrict__ maxSpeedBits, ff* __restrict__ scratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[3];  // 0, 1: matrix copies into buffer 0 (even j), 1 (odd j); 2: MMA completion
    __shared__ uint32_t tmemBase;
    __shared__ int blockList[kTcxMaxBlocks];   // matrix blocks in issue order
    __shared__ int blockCount;
    __shared__ unsigned rowMax[4][128];        // [2 tile + half][row]: largest |hi| of S (half 0) or S m (half 1)
    __shared__ int rowE[4][128];               // ... as a row exponent
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, nt = d.nt;
    const int NP = d.tcxN, KH = d.tcxKH, K = 2 * KH, passes = d.tcxPasses;
    const uint32_t aSplit = 256u * static_cast<uint32_t>(K);                                  // 128 rows x K BF16
    const uint32_t bSplit = static_cast<uint32_t>(NP >> 3) * 16u * static_cast<uint32_t>(KH); // NP rows x KH BF16
    unsigned char* A = smem_raw;                         // [slice][128][K]
    unsigned char* B = smem_raw + kTcxDigits * aSplit;   // two buffers [slice][NP][KH]
    const ff* mj = reinterpret_cast<const ff*>(d.tcxM);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcModes;
    const int nm = min(kTcModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        zspec += (size_t)member * Nz * P;
    }
    // this CTA's scratch: [mode][j][u.re u.im v.re v.im w.re w.im eta.re eta.im]
    scratch += ((size_t)member * gridDim.x + blockIdx.x) * kTcModes * Nj * 8;
    if (blockIdx.x == 0 && tid == 0 && maxSpeedBits) maxSpeedBits[member] = 0ull;
    for (int i = tid; i < 512; i += kTcThreads) rowMax[i >> 7][i & 127] = 0u;
    int derivChan[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) derivChan[d.tq[t]] = 4 + t;
    auto blockOffset = [&](int b) { return (size_t)b * kTcxDigits * bSplit; };
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init(&bars[2], 1);
        mbar_init_fence();
        // blocks (matrix, parity, pass) in the order of the tile / half / pass / parity loops
        int nb = 0;
        for (int tile = 0; tile < 2; ++tile)
            for (int half = 0; half < 2; ++half) {
                if (half == 1 && derivChan[2 * tile] < 0 && derivChan[2 * tile + 1] < 0) continue;
                const int mat = tile == 0 ? (half == 0 ? 0 : 3) : (half == 0 ? 1 : 2);
                for (int pass = 0; pass < passes; ++pass)
                    for (int par = 0; par < 2; ++par) blockList[nb++] = (mat * 2 + par) * passes + pass;
            }
        blockCount = nb;
        // the first two blocks stream in while the spectra are computed
        for (int par = 0; par < 2; ++par) {
            mbar_arrive_expect_tx(&bars[par], kTcxDigits * bSplit);
            bulk_copy_g2s(B + (size_t)par * kTcxDigits * bSplit, reinterpret_cast<const unsigned char*>(d.tcxB) + blockOffset(blockList[par]),
                          kTcxDigits * bSplit, &bars[par]);
        }
    }
    if (warp == 0) {
        tmem_alloc(&tmemBase, kTcxCols);
        tmem_relinquish();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tbase = tmemBase;

    // ---- pass 1: paired-FP32 field spectra in the stored frame (k_vinv<ff>'s
    //      arithmetic), mode-fastest so that the row-maximum atomics of a warp
    //      touch different rows
    for (int it = tid; it < nm * Nj; it += kTcThreads) {
        const int mi = it % nm, j = it / nm;
        const int mode = m0 + mi;
        const int w = d.modeWV[mode];
        const unsigned char flags = d.modeFlags[mode];
        const int idx = j + Nj * w;
        ff sf, cf;
        ff_sincos(d.omega[idx] * elapsed, sf, cf);
        const cx<ff> p = mk<ff>(cf, sf);
        auto ld = [](const double* q) { return mk<ff>(ff_from_double(q[0]), ff_from_double(q[1])); };
        const cx<ff> ap = cmul<ff>(ld(Ap + 2 * idx), p);
        const cx<ff> am = cmul<ff>(ld(Am + 2 * idx), cconj<ff>(p));
        const cx<ff> a0 = ld(A0 + 2 * idx);
        const cx<ff> uap = reinterpret_cast<const cx<ff>*>(d.fUAp)[idx];
        const cx<ff> vap = reinterpret_cast<const cx<ff>*>(d.fVAp)[idx];
        const cx<ff> wap = reinterpret_cast<const cx<ff>*>(d.fWAp)[idx];
        const cx<ff> ua0 = reinterpret_cast<const cx<ff>*>(d.fUA0)[idx];
        const cx<ff> va0 = reinterpret_cast<const cx<ff>*>(d.fVA0)[idx];
        const ff nap = reinterpret_cast<const ff*>(d.fNAp)[idx], na0 = reinterpret_cast<const ff*>(d.fNA0)[idx];
        cx<ff> f[4];
        f[0] = cadd<ff>(cadd<ff>(cmul<ff>(uap, ap), cmul<ff>(cconj<ff>(uap), am)), cmul<ff>(ua0, a0));
        f[1] = cadd<ff>(cadd<ff>(cmul<ff>(vap, ap), cmul<ff>(cconj<ff>(vap), am)), cmul<ff>(va0, a0));
        f[2] = cadd<ff>(cmul<ff>(wap, ap), cmul<ff>(wap, am));
        f[3] = mk<ff>(ap.x * nap - am.x * nap + a0.x * na0, ap.y * nap - am.y * nap + a0.y * na0);
        const ff m = mj[j];
        float4* out = reinterpret_cast<float4*>(scratch + ((size_t)mi * Nj + j) * 8);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cx<ff> v = f[q];
            if (flags & 1) v = cconj<ff>(v);
            if (flags & 2) v.y = ff(0.0f);
            out[q] = make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo);
            const int r = 4 * mi + 2 * (q & 1), t2 = 2 * (q >> 1);
            atomicMax(&rowMax[t2][r], __float_as_uint(fabsf(v.x.hi)));
            atomicMax(&rowMax[t2][r + 1], __float_as_uint(fabsf(v.y.hi)));
            atomicMax(&rowMax[t2 + 1][r], __float_as_uint(fabsf((v.x * m).hi)));
            atomicMax(&rowMax[t2 + 1][r + 1], __float_as_uint(fabsf((v.y * m).hi)));
        }
    }
    __syncthreads();
    for (int i = tid; i < 512; i += kTcThreads) rowE[i >> 7][i & 127] = tcx_row_exponent(rowMax[i >> 7][i & 127]);
    __syncthreads();

    const uint32_t idesc = idesc_bf16_f32(128, NP);
    const uint32_t sA = smem_u32(A), sB = smem_u32(B);
    uint32_t phaseM = 0;
    int bi = 0;  // index of the current matrix block in blockList
    for (int tile = 0; tile < 2; ++tile) {
        for (int half = 0; half < 2; ++half) {
            // z-derivatives only where a flux target needs them
            if (half == 1 && derivChan[2 * tile] < 0 && derivChan[2 * tile + 1] < 0) continue;
            const int mat = tile == 0 ? (half == 0 ? 0 : 3) : (half == 0 ? 1 : 2);  // Ccos, -Csin | Csin, Ccos
            const int rt = 2 * tile + half;
            // ---- A: six digit slices of the rows (mode, u|v or w|eta, re|im) of S
            //      (values) or S m (z-derivatives), K = even j then odd j; absent
            //      modes and the K padding stay zero.  Every thread has seen the
            //      previous block's MMAs complete.
            for (uint32_t i = tid; i < kTcxDigits * aSplit / 16; i += kTcThreads)
                reinterpret_cast<uint4*>(A)[i] = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            for (int it = tid; it < nm * Nj; it += kTcThreads) {
                const int mi = it / Nj, j = it - mi * Nj;
                const float4* src = reinterpret_cast<const float4*>(scratch + ((size_t)mi * Nj + j) * 8) + 2 * tile;
                const float4 v0 = src[0], v1 = src[1];
                ff vals[4] = {ff(v0.x, v0.y), ff(v0.z, v0.w), ff(v1.x, v1.y), ff(v1.z, v1.w)};
                if (half == 1) {
                    const ff m = mj[j];
#pragma unroll
                    for (int k = 0; k < 4; ++k) vals[k] = vals[k] * m;
                }
                const int kk = (j & 1) ? KH + (j >> 1) : (j >> 1);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int r = 4 * mi + k;
                    unsigned short dg[kTcxDigits];
                    tcx_digits(vals[k], rowE[rt][r], dg);
                    const uint32_t off = tc_kmajor_offset(r, kk, K);
#pragma unroll
                    for (int s = 0; s < kTcxDigits; ++s) *reinterpret_cast<unsigned short*>(A + s * aSplit + off) = dg[s];
                }
            }
            fence_proxy_async_smem();
            __syncthreads();

            for (int pass = 0; pass < passes; ++pass) {
                // ---- matrix blocks bi (even j) and bi + 1 (odd j) of (mat, pass), prefetched
                //      into buffers 0 and 1: 2 x 21 digit products, one completion wait
                if (tid == 0) {
                    for (int par = 0; par < 2; ++par) {
                        const uint32_t sBb = sB + static_cast<uint32_t>(par) * kTcxDigits * bSplit;
                        if (!mbar_wait(&bars[par], static_cast<uint32_t>(bi >> 1) & 1u, d.status)) continue;
                        tc_fence_after_sync();
                        uint32_t started = 0u;  // bit a: accumulator a holds a partial sum
                        for (int k0 = 0; k0 < KH; k0 += 16) {
                            const uint32_t aK = static_cast<uint32_t>((par * KH + k0) >> 3) * 128u;
                            const uint32_t bK = static_cast<uint32_t>(k0 >> 3) * 128u;
                            for (int lv = 5; lv >= 0; --lv) {  // smallest level first
                                const int acc = lv < 3 ? lv : 3;
                                const uint32_t tcol = tbase + static_cast<uint32_t>((par * 4 + acc) * NP);
                                for (int s = 0; s <= lv; ++s) {
                                    const int t = lv - s;
                                    const uint64_t ad = smem_desc_noswizzle(sA + static_cast<uint32_t>(s) * aSplit + aK, 128u, 16u * K);
                                    const uint64_t bd = smem_desc_noswizzle(sBb + static_cast<uint32_t>(t) * bSplit + bK, 128u, 16u * KH);
                                    tc_mma_bf16(tcol, ad, bd, idesc, (started >> acc) & 1u);
                                    started |= 1u << acc;
                                }
                            }
                        }
                    }
                    tc_commit(&bars[2]);
                }
                bi += 2;
                mbar_wait(&bars[2], phaseM, d.status);  // MMAs done: accumulators final, both buffers free
                phaseM ^= 1u;
                tc_fence_after_sync();
                // the next pair of blocks streams in during the drain (and the next assembly)
                if (tid == 0 && bi < blockCount) {
                    for (int par = 0; par < 2; ++par) {
                        mbar_arrive_expect_tx(&bars[par], kTcxDigits * bSplit);
                        bulk_copy_g2s(B + (size_t)par * kTcxDigits * bSplit,
                                      reinterpret_cast<const unsigned char*>(d.tcxB) + blockOffset(blockList[bi + par]),
                                      kTcxDigits * bSplit, &bars[par]);
                    }
                }

                // ---- drain: row r = 32 (warp % 4) + lane; out[n] = E + O, out[Nz-1-n] = E - O
                //      (cosine) or O - E (sine), E and O the sums of each parity's accumulators
                {
                    const int quarter = warp & 3, cgroup = warp >> 2;
                    const int r = 32 * quarter + lane;
                    const int mi = r >> 2, fl = (r >> 1) & 1, part = r & 1;
                    const bool valid = mi < nm;
                    const int mode = m0 + (valid ? mi : 0);
                    const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
                    const int Er = rowE[rt][r];
                    int ch;
                    bool sine;
                    if (tile == 0) { ch = half == 0 ? fl : derivChan[fl]; sine = half == 1; }
                    else { ch = half == 0 ? 2 + fl : derivChan[2 + fl]; sine = half == 0; }
                    const int* Fx = d.tcxF + (static_cast<size_t>(mat) * passes + pass) * NP;
                    const uint32_t rowAddr = tbase + (static_cast<uint32_t>(32 * quarter) << 16);
                    ff2* base = zspec + (size_t)(ch < 0 ? 0 : ch) * d.zTotal * P;
                    const int nCols = min(NP, Zh - pass * NP);  // columns beyond zHalf carry no output
                    for (int c0 = 4 * cgroup; c0 < nCols; c0 += 16) {
                        float e[4][4], o[4][4];
#pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            tc_ld_32x32b_x4(rowAddr + static_cast<uint32_t>(a * NP + c0), e[a]);
                            tc_ld_32x32b_x4(rowAddr + static_cast<uint32_t>((4 + a) * NP + c0), o[a]);
                        }
                        tc_wait_ld();
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int n = pass * NP + c0 + i;
                            const int ex = Er + Fx[c0 + i];
                            const ff E = tcx_combine(e[0][i], e[1][i], e[2][i], e[3][i], ex);
                            const ff O = tcx_combine(o[0][i], o[1][i], o[2][i], o[3][i], ex);
                            const ff lo = E + O;
                            const ff hi = sine ? O - E : E - O;
                            const float loH = __shfl_xor_sync(0xffffffffu, lo.hi, 1), loL = __shfl_xor_sync(0xffffffffu, lo.lo, 1);
                            const float hiH = __shfl_xor_sync(0xffffffffu, hi.hi, 1), hiL = __shfl_xor_sync(0xffffffffu, hi.lo, 1);
                            if (part == 0 && valid && ch >= 0 && n < Zh) {
                                ff2 v;
                                v.x = lo; v.y = ff(loH, loL);
                                base[(size_t)n * P + pos] = v;
                                if (cpos >= 0) { v.y = -v.y; base[(size_t)n * P + cpos] = v; }
                                const int n2 = Nz - 1 - n;
                                if (n2 != n) {
                                    v.x = hi; v.y = ff(hiH, hiL);
                                    base[(size_t)n2 * P + pos] = v;
                                    if (cpos >= 0) { v.y = -v.y; base[(size_t)n2 * P + cpos] = v; }
                                }
                            }
                        }
                    }
                }
                tc_fence_before_sync();
                __syncthreads();  // tensor-memory reads done before the next block's MMAs
                tc_fence_after_sync();
            }
        }
    }
    if (warp == 0) tmem_dealloc(tbase, kTcxCols);
}

}  // namespace dev
}  // namespace wvgpu

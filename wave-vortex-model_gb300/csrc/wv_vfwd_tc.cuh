// Vertical forward transform of the mixed-form flux on the tensor cores
// (tcgen05.mma, FP32 accumulators in tensor memory): the forward DCT-I / DST-I
// with its normalization (normalizeForwardDCT / DST, kernel.cpp:176-193) of the
// product spectra, as split-BF16 GEMMs, and the folded FP32 projection of the
// transformed targets in the tensor-memory drain.
//
// One CTA (16 warps) takes 32 retained columns and runs two tiles of M = 128
// rows (mode, target, re|im): tile 0 the cosine-family targets u, v, tile 1 the
// sine-family targets w, eta.  Folding z with Nz-1-z gives P_n = S_n + S_{Nz-1-n}
// and Q_n = S_n - S_{Nz-1-n} (n < Zh; P = Q = S at a middle point); even output
// j take P (cosine) or Q (sine), odd j the other one, so each tile runs two
// GEMMs over K = n into two accumulators:
//   cosine: D_even = A_P x Fcos_even^T,  D_odd = A_Q x Fcos_odd^T
//   sine:   D_even = A_Q x Fsin_even^T,  D_odd = A_P x Fsin_odd^T
// with every FP32 operand split into three BF16 pieces and the six leading
// cross products accumulated smallest first (FP32 precision, as k_vinv_tc).
// The four accumulators (two per family) stay in tensor memory until both tiles
// are done; the drain then projects every (mode, j) with the arithmetic of
// k_vfwd's mixed branch and stores the flux.
#pragma once

#include "wv_kernels.cuh"
#include "wv_tc.cuh"
#include "wv_vinv_tc.cuh"

namespace wvgpu {
namespace dev {

constexpr uint32_t kTcFwdCols = 512;  // tensor-memory columns: four accumulators of NF <= 128

// Eight consecutive K values of one row as three BF16 pieces: one 16-byte store per piece.
__device__ __forceinline__ void put_split3_run8(unsigned char* A, uint32_t split, uint32_t off, const float (&x)[8]) {
    uint32_t h[4], m[4], l[4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        uint32_t hh[2], mm[2], ll[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float b0, b1, b2;
            hh[k] = bf16_bits(x[i + k], b0);
            const float r1 = x[i + k] - b0;
            mm[k] = bf16_bits(r1, b1);
            ll[k] = bf16_bits(r1 - b1, b2);
        }
        h[i >> 1] = hh[0] | (hh[1] << 16);
        m[i >> 1] = mm[0] | (mm[1] << 16);
        l[i >> 1] = ll[0] | (ll[1] << 16);
    }
    *reinterpret_cast<uint4*>(A + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(A + split + off) = make_uint4(m[0], m[1], m[2], m[3]);
    *reinterpret_cast<uint4*>(A + 2 * split + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

// Element k of four registers (k in 0..3, lane-dependent) without local memory.
__device__ __forceinline__ float pick4(const float* v, int k) {
    const float a = (k & 1) ? v[1] : v[0];
    const float b = (k & 1) ? v[3] : v[2];
    return (k & 2) ? b : a;
}

// Tensor-memory drain of one output parity: lanes 4 m .. 4 m + 3 hold, for
// mode m and 16 outputs j, the (u.re, u.im, v.re, v.im) rows of the cosine
// accumulator (a) and the (w.re, w.im, eta.re, eta.im) rows of the sine
// accumulator (b).  A 4 x 4 transpose per group of four columns (rotating
// shuffles) hands lane 4 m + s the eight values of column 4 g + s, which it
// projects and stores.
__device__ __forceinline__ void vfwd_tc_project(const DescDev& d, const float (&a)[16], const float (&b)[16], int c0,
                                                int parity, int mode, bool valid, double elapsed, double maxSpeed,
                                                int applyDamping, const double* Ap, const double* Am, const double* A0,
                                                double* Fp, double* Fm, double* F0) {
    const int lane = threadIdx.x & 31, sub = lane & 3, base = lane & ~3;
    const int Nj = d.Nj;
    const int w = d.modeWV[mode];
    const bool conj = d.modeFlags[mode] & 1;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        float ca[4], cb[4];  // ca[k] / cb[k]: row k of the group at column 4 g + sub
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // round r: read lane (sub + r) & 3 its value for column 4 g + sub, i.e. every
            // lane sends its value for column 4 g + ((sub - r) & 3)
            const int sendCol = (sub - r) & 3;
            const float va = __shfl_sync(0xffffffffu, pick4(a + 4 * g, sendCol), base + ((sub + r) & 3));
            const float vb = __shfl_sync(0xffffffffu, pick4(b + 4 * g, sendCol), base + ((sub + r) & 3));
            const int k = (sub + r) & 3;
            // static register targets: k is lane-dependent, so select into each slot
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (k == t) { ca[t] = va; cb[t] = vb; }
            }
        }
        const int j = 2 * (c0 + 4 * g + sub) + parity;
        if (valid && j < Nj) {
            const float sg = conj ? -1.f : 1.f;
            const float2 ch[4] = {make_float2(ca[0], sg * ca[1]), make_float2(ca[2], sg * ca[3]),
                                  make_float2(cb[0], sg * cb[1]), make_float2(cb[2], sg * cb[3])};
            mixed_project_store(d, j + Nj * w, w, j, ch, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
        }
    }
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_vfwd_tc(DescDev d, const float2* __restrict__ fspec, double elapsed, const double* __restrict__ Ap,
          const double* __restrict__ Am, const double* __restrict__ A0, const unsigned long long* __restrict__ maxSpeedBits,
          int applyDamping, double* __restrict__ Fp, double* __restrict__ Fm, double* __restrict__ F0) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];  // 0: matrix copies, 1: MMA completion
    __shared__ uint32_t tmemBase;
    const int Nz = d.Nz, Zh = d.zHalf, P = d.positions;
    const int NF = d.tcFN, KF = d.tcFK;
    const uint32_t aSplit = 256u * static_cast<uint32_t>(KF);                                  // 128 rows x KF BF16
    const uint32_t bSplit = static_cast<uint32_t>(NF >> 3) * 16u * static_cast<uint32_t>(KF);  // NF rows x KF BF16
    unsigned char* A = smem_raw;                 // [variant P|Q][piece][128][KF]
    unsigned char* B = smem_raw + 6 * aSplit;    // [parity even|odd][piece][NF][KF]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcModes;
    const int nm = min(kTcModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        Fp += o; Fm += o; F0 += o;
        fspec += (size_t)member * Nz * P;
    }
    int chanOf[4] = {-1, -1, -1, -1};
    for (int c = 0; c < d.nt; ++c) chanOf[d.tq[c]] = c;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init_fence();
    }
    if (warp == 0) {
        tmem_alloc(&tmemBase, kTcFwdCols);
        tmem_relinquish();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tbase = tmemBase;
    const uint32_t idesc = idesc_bf16_f32(128, NF);
    const uint32_t sA = smem_u32(A), sB = smem_u32(B);
    uint32_t phaseB = 0, phaseM = 0;
    for (int tile = 0; tile < 2; ++tile) {
        // matrices of this family (even and odd rows, three pieces each): one bulk copy
        if (tid == 0) {
            mbar_arrive_expect_tx(&bars[0], 6 * bSplit);
            bulk_copy_g2s(B, reinterpret_cast<const unsigned char*>(d.tcFB) + (size_t)tile * 6 * bSplit, 6 * bSplit, &bars[0]);
        }
        // A operands P and Q of the tile's two targets, split into BF16 pieces.  One
        // item = one row r = 4 mi + 2 tp + part and 8 consecutive n (one 16-byte run
        // of each piece); the low three bits of the item index walk the eight rows
        // of a core matrix, so the eight lanes of each store phase hit eight
        // different 16-byte bank groups.  Rows of absent targets or modes and the
        // K padding are written as zeros.  (For the second tile, every thread has
        // seen the first tile's MMAs complete, so A is free.)
        {
            const int nb8 = KF >> 3;
            for (int it = tid; it < 128 * nb8; it += kTcThreads) {
                const int part = it & 1, tp = (it >> 1) & 1, miLo = (it >> 2) & 1;
                const int rest = it >> 3;
                const int mi = 2 * (rest & 15) + miLo, nb = rest >> 4;
                const int c = chanOf[2 * tile + tp];
                float vp[8], vq[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) { vp[i] = 0.f; vq[i] = 0.f; }
                if (c >= 0 && mi < nm) {
                    const int pos = d.modePos[m0 + mi];
                    const float* col = reinterpret_cast<const float*>(fspec + (size_t)c * d.zTotal * P + pos) + part;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int n = 8 * nb + i;
                        if (n < Zh) {
                            const int n2 = Nz - 1 - n;
                            const float a = col[(size_t)n * P * 2];
                            if (n2 != n) {
                                const float b = col[(size_t)n2 * P * 2];
                                vp[i] = a + b;
                                vq[i] = a - b;
                            } else {
                                vp[i] = a;
                                vq[i] = a;
                            }
                        }
                    }
                }
                const uint32_t off = tc_kmajor_offset(4 * mi + 2 * tp + part, 8 * nb, KF);
                put_split3_run8(A, aSplit, off, vp);
                put_split3_run8(A + 3 * aSplit, aSplit, off, vq);
            }
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (mbar_wait(&bars[0], phaseB, d.status)) {
                tc_fence_after_sync();
                const int pa[6] = {2, 1, 0, 1, 0, 0};
                const int pb[6] = {0, 1, 2, 0, 1, 0};
                for (int acc = 0; acc < 2; ++acc) {
                    // cosine: even <- P, odd <- Q;  sine: even <- Q, odd <- P
                    const int variant = (tile == 0) ? acc : 1 - acc;
                    const uint32_t sAv = sA + static_cast<uint32_t>(variant) * 3u * aSplit;
                    const uint32_t sBp = sB + static_cast<uint32_t>(acc) * 3u * bSplit;
                    const uint32_t tcol = tbase + static_cast<uint32_t>((2 * tile + acc) * NF);
                    uint32_t accumulate = 0;
                    for (int k0 = 0; k0 < KF; k0 += 16) {
                        for (int p = 0; p < 6; ++p) {
                            const uint64_t ad = smem_desc_noswizzle(sAv + pa[p] * aSplit + static_cast<uint32_t>(k0 >> 3) * 128u, 128u,
                                                                    16u * KF);
                            const uint64_t bd = smem_desc_noswizzle(sBp + pb[p] * bSplit + static_cast<uint32_t>(k0 >> 3) * 128u, 128u,
                                                                    16u * KF);
                            tc_mma_bf16(tcol, ad, bd, idesc, accumulate);
                            accumulate = 1;
                        }
                    }
                }
            }
            tc_commit(&bars[1]);
        }
        phaseB ^= 1u;
        mbar_wait(&bars[1], phaseM, d.status);  // MMAs done: A and B are free for the next tile
        phaseM ^= 1u;
        tc_fence_after_sync();
    }
    // drain: row r = 32 (warp % 4) + lane holds (mode r / 4, target pair, re|im) of both
    // families; the four warps of a lane quarter split the column chunks
    {
        const int quarter = warp & 3, cgroup = warp >> 2;
        const int r = 32 * quarter + lane;
        const int mi = r >> 2;
        const bool valid = mi < nm;
        const int mode = m0 + (valid ? mi : 0);
        const double maxSpeed = applyDamping ? __longlong_as_double((long long)maxSpeedBits[member]) : 0.0;
        const uint32_t rowAddr = tbase + (static_cast<uint32_t>(32 * quarter) << 16);
        for (int c0 = 16 * cgroup; c0 < NF; c0 += 64) {
            for (int parity = 0; parity < 2; ++parity) {
                float a[16], b[16];
                tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>(parity * NF + c0), a);
                tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>((2 + parity) * NF + c0), b);
                tc_wait_ld();
                vfwd_tc_project(d, a, b, c0, parity, mode, valid, elapsed, maxSpeed, applyDamping, Ap, Am, A0, Fp, Fm, F0);
            }
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    if (warp == 0) tmem_dealloc(tbase, kTcFwdCols);
}

}  // namespace dev
}  // namespace wvgpu

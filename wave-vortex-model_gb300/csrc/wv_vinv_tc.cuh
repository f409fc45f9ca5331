// Vertical inverse transform of the mixed-form flux on the tensor cores
// (tcgen05.mma, FP32 accumulators in tensor memory).
//
// Same result as k_vinv<float, true> (phase, field spectra, folded vertical
// inverse DCT-I / DST-I, z-derivatives of the flux targets) with the dense
// contraction done as split-BF16 GEMMs.  One CTA (16 warps) takes 32 retained
// columns ("modes"), assembles their four field spectra once, and runs two
// tiles of M = 128 rows:
//   tile 0: rows (mode, u|v, re|im) against Ccos (values) and CsinM (d/dz)
//   tile 1: rows (mode, w|eta, re|im) against Csin (values) and CcosM (d/dz)
// The z <-> Nz-1-z fold splits K into even j (columns 0..KE) and odd j
// (KE..K); each half accumulates into its own tensor-memory accumulator
// (D_E, D_O) with N = Zh rounded up to 16, and out[n] = E + O,
// out[Nz-1-n] = E - O (cosine family) or O - E (sine family).
// Each FP32 operand is split into three BF16 pieces (24 significant bits) and
// the six leading cross products are accumulated, smallest first, so the
// contraction keeps FP32 precision.  The matrices are pre-split on the host in
// the canonical no-swizzle K-major layout (8-row x 16-byte core matrices,
// 128 bytes apart along K, 16 K bytes apart along M/N) and staged with one bulk
// copy per matrix; the A operand is written by the CTA in the same layout.
#pragma once

#include <cuda_bf16.h>

#include "wv_kernels.cuh"
#include "wv_tc.cuh"

namespace wvgpu {
namespace dev {

constexpr int kTcModes = 32;        // retained columns per CTA (M = 128 rows = 32 modes x 2 fields x re/im)
constexpr int kTcThreads = 512;     // 16 warps; warp w drains tensor-memory lanes 32 (w % 4) .. + 31, column chunks w / 4, + 4, ...
constexpr uint32_t kTcCols = 512;   // tensor-memory columns allocated (4 accumulators of N <= 128)

// Byte offset of element (row r, k) in a canonical no-swizzle K-major tile with K columns.
__host__ __device__ inline uint32_t tc_kmajor_offset(int r, int k, int K) {
    return static_cast<uint32_t>(r >> 3) * (16u * K) + static_cast<uint32_t>(k >> 3) * 128u + static_cast<uint32_t>(r & 7) * 16u +
           static_cast<uint32_t>(k & 7) * 2u;
}

// x as hi + mid + lo BF16 pieces (each the rounded remainder of the previous).
__device__ __forceinline__ void put_split3(unsigned char* A, uint32_t split, uint32_t off, float x) {
    float b0, b1, b2;
    const unsigned short h = bf16_bits(x, b0);
    const float r1 = x - b0;
    const unsigned short m = bf16_bits(r1, b1);
    const float r2 = r1 - b1;
    const unsigned short l = bf16_bits(r2, b2);
    *reinterpret_cast<unsigned short*>(A + off) = h;
    *reinterpret_cast<unsigned short*>(A + split + off) = m;
    *reinterpret_cast<unsigned short*>(A + 2 * split + off) = l;
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_vinv_tc(DescDev d, const double* __restrict__ Ap, const double* __restrict__ Am, const double* __restrict__ A0,
          double elapsed, float2* __restrict__ zspec, unsigned long long* __restrict__ maxSpeedBits) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];  // 0: matrix copies, 1: MMA completion
    __shared__ uint32_t tmemBase;
    __shared__ int aborted;  // a bounded operand wait ran out: no further MMA, no drain
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, nt = d.nt;
    const int NP = d.tcN, KE = d.tcKE, K = d.tcK;
    const uint32_t aSplit = 256u * static_cast<uint32_t>(K);                                  // 128 rows x K BF16
    const uint32_t bSplit = static_cast<uint32_t>(NP >> 3) * 16u * static_cast<uint32_t>(K);  // NP rows x K BF16
    // A operands of both tiles (3 pieces each), then the B operand (3 pieces of one matrix)
    unsigned char* A = smem_raw;
    unsigned char* B = smem_raw + 6 * aSplit;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcModes;
    const int nm = min(kTcModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) {
        const long long o = member * d.memberStride;
        Ap += o; Am += o; A0 += o;
        zspec += (size_t)member * Nz * P;
    }
    if (blockIdx.x == 0 && tid == 0 && maxSpeedBits) maxSpeedBits[member] = 0ull;
    for (uint32_t i = tid; i < 6 * aSplit / 16; i += kTcThreads) reinterpret_cast<uint4*>(A)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_init_fence();
        aborted = 0;
    }
    if (warp == 0) {
        tmem_alloc(&tmemBase, kTcCols);
        tmem_relinquish();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tbase = tmemBase;
    const uint32_t idesc = idesc_bf16_f32(128, NP);
    const uint32_t sA = smem_u32(A), sB = smem_u32(B);
    int derivChan[4] = {-1, -1, -1, -1};
    for (int t = 0; t < nt; ++t) derivChan[d.tq[t]] = 4 + t;

    // ---- A operands: the four field spectra of every (mode, j), split into BF16 pieces;
    //      tile 0 rows (mode, u|v, re|im), tile 1 rows (mode, w|eta, re|im)
    for (int it = tid; it < nm * Nj; it += kTcThreads) {
        const int mi = it / Nj, j = it - mi * Nj;
        const int mode = m0 + mi;
        const int w = d.modeWV[mode];
        const unsigned char flags = d.modeFlags[mode];
        const int idx = j + Nj * w;
        const double ang = d.omega[idx] * elapsed;
        const double red = ang - 6.283185307179586476925 * rint(ang * 0.15915494309189533577);
        float sf, cf;
        sincosf(float(red), &sf, &cf);
        const float2 ap0 = make_float2(float(Ap[2 * idx]), float(Ap[2 * idx + 1]));
        const float2 am0 = make_float2(float(Am[2 * idx]), float(Am[2 * idx + 1]));
        const float2 a0 = make_float2(float(A0[2 * idx]), float(A0[2 * idx + 1]));
        const float2 ap = make_float2(ap0.x * cf - ap0.y * sf, ap0.x * sf + ap0.y * cf);
        const float2 am = make_float2(am0.x * cf + am0.y * sf, am0.y * cf - am0.x * sf);
        auto cm2 = [](float2 x, float2 y) { return make_float2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x); };
        auto cj = [](float2 x) { return make_float2(x.x, -x.y); };
        auto ca = [](float2 x, float2 y) { return make_float2(x.x + y.x, x.y + y.y); };
        const float2 uap = *reinterpret_cast<const float2*>(d.fUAp + 2 * idx);
        const float2 vap = *reinterpret_cast<const float2*>(d.fVAp + 2 * idx);
        const float2 wap = *reinterpret_cast<const float2*>(d.fWAp + 2 * idx);
        const float2 ua0 = *reinterpret_cast<const float2*>(d.fUA0 + 2 * idx);
        const float2 va0 = *reinterpret_cast<const float2*>(d.fVA0 + 2 * idx);
        const float nap = d.fNAp[idx], na0 = d.fNA0[idx];
        float2 f[4];
        f[0] = ca(ca(cm2(uap, ap), cm2(cj(uap), am)), cm2(ua0, a0));
        f[1] = ca(ca(cm2(vap, ap), cm2(cj(vap), am)), cm2(va0, a0));
        f[2] = ca(cm2(wap, ap), cm2(wap, am));
        f[3] = make_float2(ap.x * nap - am.x * nap + a0.x * na0, ap.y * nap - am.y * nap + a0.y * na0);
        const int kk = (j & 1) ? KE + (j >> 1) : (j >> 1);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float2 v = f[q];
            if (flags & 1) v = cj(v);
            if (flags & 2) v.y = 0.f;
            unsigned char* At = A + (q >> 1) * 3 * aSplit;
            put_split3(At, aSplit, tc_kmajor_offset(4 * mi + 2 * (q & 1) + 0, kk, K), v.x);
            put_split3(At, aSplit, tc_kmajor_offset(4 * mi + 2 * (q & 1) + 1, kk, K), v.y);
        }
    }
    fence_proxy_async_smem();
    __syncthreads();

    uint32_t phaseB = 0, phaseM = 0;
    for (int tile = 0; tile < 2 && !aborted; ++tile) {
        const uint32_t sAt = sA + static_cast<uint32_t>(tile) * 3u * aSplit;
        // ---- value matrix (half 0), then z-derivative matrix (half 1)
        for (int half = 0; half < 2; ++half) {
            const int mat = tile == 0 ? (half == 0 ? 0 : 3) : (half == 0 ? 1 : 2);  // Ccos, CsinM | Csin, CcosM
            if (tid == 0) {
                // test hook: the first operand wait gets no copy, so it runs out before any MMA
                const bool inject = d.injectWaitPolls != 0 && tile == 0 && half == 0;
                if (!inject) {
                    mbar_arrive_expect_tx(&bars[0], 3 * bSplit);
                    bulk_copy_g2s(B, reinterpret_cast<const unsigned char*>(d.tcB) + (size_t)mat * 3 * bSplit, 3 * bSplit, &bars[0]);
                }
                const bool landed = inject ? mbar_wait_polls(&bars[0], phaseB, d.status, d.injectWaitPolls)
                                           : mbar_wait(&bars[0], phaseB, d.status);
                if (!landed) {
                    // a copy that was issued is waited for (bounded) before B is reused or
                    // the CTA exits; then this CTA issues no MMA and releases its waiters
                    if (!inject) mbar_wait(&bars[0], phaseB, nullptr);
                    aborted = 1;
                    mbar_arrive(&bars[1]);
                } else {
                    tc_fence_after_sync();
                    // pieces (a, b), smallest products first
                    const int pa[6] = {2, 1, 0, 1, 0, 0};
                    const int pb[6] = {0, 1, 2, 0, 1, 0};
                    for (int acc = 0; acc < 2; ++acc) {
                        const int kBeg = acc == 0 ? 0 : KE, kEnd = acc == 0 ? KE : K;
                        const uint32_t tcol = tbase + static_cast<uint32_t>((2 * half + acc) * NP);
                        uint32_t accumulate = 0;
                        for (int k0 = kBeg; k0 < kEnd; k0 += 16) {
                            for (int p = 0; p < 6; ++p) {
                                const uint64_t ad = smem_desc_noswizzle(sAt + pa[p] * aSplit + static_cast<uint32_t>(k0 >> 3) * 128u,
                                                                        128u, 16u * K);
                                const uint64_t bd = smem_desc_noswizzle(sB + pb[p] * bSplit + static_cast<uint32_t>(k0 >> 3) * 128u,
                                                                        128u, 16u * K);
                                tc_mma_bf16(tcol, ad, bd, idesc, accumulate);
                                accumulate = 1;
                            }
                        }
                    }
                    tc_commit(&bars[1]);
                }
            }
            phaseB ^= 1u;
            mbar_wait(&bars[1], phaseM, d.status);  // MMAs done: B is free, accumulators are final
            phaseM ^= 1u;
            tc_fence_after_sync();
            __syncthreads();  // every thread sees `aborted`
            if (aborted) break;
        }
        if (aborted) break;

        // ---- drain: row r = 32 (warp % 4) + lane; the four warps of a lane quarter split the column chunks
        {
            const int quarter = warp & 3, cgroup = warp >> 2;
            const int r = 32 * quarter + lane;
            const int mi = r >> 2, fl = (r >> 1) & 1, part = r & 1;
            const bool valid = mi < nm;
            const int mode = m0 + (valid ? mi : 0);
            const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
            const uint32_t rowAddr = tbase + (static_cast<uint32_t>(32 * quarter) << 16);
            for (int half = 0; half < 2; ++half) {
                int ch;
                bool sine;
                if (tile == 0) { ch = half == 0 ? fl : derivChan[fl]; sine = half == 1; }
                else { ch = half == 0 ? 2 + fl : derivChan[2 + fl]; sine = half == 0; }
                for (int c0 = 16 * cgroup; c0 < NP; c0 += 64) {
                    float e[16], o[16];
                    tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>((2 * half) * NP + c0), e);
                    tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>((2 * half + 1) * NP + c0), o);
                    tc_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const float lo = e[i] + o[i];
                        const float hi = sine ? o[i] - e[i] : e[i] - o[i];
                        const float loP = __shfl_xor_sync(0xffffffffu, lo, 1);
                        const float hiP = __shfl_xor_sync(0xffffffffu, hi, 1);
                        const int n = c0 + i;
                        if (part == 0 && valid && ch >= 0 && n < Zh) {
                            float2* base = zspec + (size_t)ch * d.zTotal * P;
                            base[(size_t)n * P + pos] = make_float2(lo, loP);
                            if (cpos >= 0) base[(size_t)n * P + cpos] = make_float2(lo, -loP);
                            const int n2 = Nz - 1 - n;
                            if (n2 != n) {
                                base[(size_t)n2 * P + pos] = make_float2(hi, hiP);
                                if (cpos >= 0) base[(size_t)n2 * P + cpos] = make_float2(hi, -hiP);
                            }
                        }
                    }
                }
            }
        }
        tc_fence_before_sync();
        __syncthreads();  // all tensor-memory reads done before the next tile's MMAs
        tc_fence_after_sync();
    }
    if (warp == 0) tmem_dealloc(tbase, kTcCols);
}

}  // namespace dev
}  // namespace wvgpu

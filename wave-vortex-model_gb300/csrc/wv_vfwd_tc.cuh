// Vertical forward transform of the mixed-form flux on the tensor cores
// (tcgen05.mma, FP32 accumulators in tensor memory): the forward DCT-I / DST-I
// with its normalization (normalizeForwardDCT / DST, kernel.cpp:176-193) of the
// product spectra, as split-BF16 GEMMs, then the folded FP32 projection in a
// second pass (k_vfwd_proj).
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
// The transformed values go to vspec[q][member][idx] (FP32 complex, canonical
// (mode, j) order) and k_vfwd_proj applies the projection of k_vfwd's mixed
// branch per (mode, j).
#pragma once

#include "wv_kernels.cuh"
#include "wv_tc.cuh"
#include "wv_vinv_tc.cuh"

namespace wvgpu {
namespace dev {

constexpr uint32_t kTcFwdCols = 256;  // tensor-memory columns: two accumulators of NF <= 128

__global__ void __launch_bounds__(kTcThreads, 1)
k_vfwd_tc(DescDev d, const float2* __restrict__ fspec, float2* __restrict__ vspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];  // 0: matrix copies, 1: MMA completion
    __shared__ uint32_t tmemBase;
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, M = d.M;
    const int NF = d.tcFN, KF = d.tcFK;
    const uint32_t aSplit = 256u * static_cast<uint32_t>(KF);                                  // 128 rows x KF BF16
    const uint32_t bSplit = static_cast<uint32_t>(NF >> 3) * 16u * static_cast<uint32_t>(KF);  // NF rows x KF BF16
    unsigned char* A = smem_raw;                 // [variant P|Q][piece][128][KF]
    unsigned char* B = smem_raw + 6 * aSplit;    // [parity even|odd][piece][NF][KF]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTcModes;
    const int nm = min(kTcModes, d.Nkl - m0);
    const int member = blockIdx.y;
    if (member > 0) fspec += (size_t)member * Nz * P;
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
        // A operands P and Q of the tile's two targets, split into BF16 pieces
        for (uint32_t i = tid; i < 6 * aSplit / 16; i += kTcThreads) reinterpret_cast<uint4*>(A)[i] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();
        for (int it = tid; it < 2 * Zh * nm; it += kTcThreads) {
            const int mi = it % nm;
            const int rest = it / nm;
            const int n = rest % Zh, tp = rest / Zh;
            const int c = chanOf[2 * tile + tp];
            if (c < 0) continue;
            const int pos = d.modePos[m0 + mi];
            const float2* col = fspec + (size_t)c * d.zTotal * P + pos;
            const float2 a = col[(size_t)n * P];
            const int n2 = Nz - 1 - n;
            float2 vp = a, vq = a;
            if (n2 != n) {
                const float2 b = col[(size_t)n2 * P];
                vp = make_float2(a.x + b.x, a.y + b.y);
                vq = make_float2(a.x - b.x, a.y - b.y);
            }
            const int r = 4 * mi + 2 * tp;
            put_split3(A, aSplit, tc_kmajor_offset(r, n, KF), vp.x);
            put_split3(A, aSplit, tc_kmajor_offset(r + 1, n, KF), vp.y);
            put_split3(A + 3 * aSplit, aSplit, tc_kmajor_offset(r, n, KF), vq.x);
            put_split3(A + 3 * aSplit, aSplit, tc_kmajor_offset(r + 1, n, KF), vq.y);
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
                    const uint32_t tcol = tbase + static_cast<uint32_t>(acc * NF);
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
        mbar_wait(&bars[1], phaseM, d.status);  // MMAs done: A and B are free, accumulators final
        phaseM ^= 1u;
        tc_fence_after_sync();
        // drain: row r = 32 (warp % 4) + lane; the four warps of a lane quarter split the column chunks
        {
            const int quarter = warp & 3, cgroup = warp >> 2;
            const int r = 32 * quarter + lane;
            const int mi = r >> 2, tp = (r >> 1) & 1, part = r & 1;
            const int q = 2 * tile + tp;
            const bool valid = mi < nm && chanOf[q] >= 0;
            const int mode = m0 + (mi < nm ? mi : 0);
            const int w = d.modeWV[mode];
            const bool conj = d.modeFlags[mode] & 1;
            const uint32_t rowAddr = tbase + (static_cast<uint32_t>(32 * quarter) << 16);
            float2* out = vspec + ((size_t)q * d.members + member) * M;
            for (int c0 = 16 * cgroup; c0 < NF; c0 += 64) {
                float e[16], o[16];
                tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>(c0), e);
                tc_ld_32x32b_x16(rowAddr + static_cast<uint32_t>(NF + c0), o);
                tc_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float eP = __shfl_xor_sync(0xffffffffu, e[i], 1);
                    const float oP = __shfl_xor_sync(0xffffffffu, o[i], 1);
                    const int je = 2 * (c0 + i), jo = je + 1;
                    if (part == 0 && valid) {
                        if (je < Nj) out[je + Nj * w] = make_float2(e[i], conj ? -eP : eP);
                        if (jo < Nj) out[jo + Nj * w] = make_float2(o[i], conj ? -oP : oP);
                    }
                }
            }
        }
        tc_fence_before_sync();
        __syncthreads();  // all tensor-memory reads done before the next tile's MMAs
        tc_fence_after_sync();
    }
    if (warp == 0) tmem_dealloc(tbase, kTcFwdCols);
}

// Projection of the tensor-core forward transform's output: one thread per
// (member, mode, j), the same arithmetic as k_vfwd's mixed branch.
__global__ void __launch_bounds__(256) k_vfwd_proj(DescDev d, const float2* __restrict__ vspec, double elapsed,
                                                  const double* __restrict__ Ap, const double* __restrict__ Am,
                                                  const double* __restrict__ A0,
                                                  const unsigned long long* __restrict__ maxSpeedBits, int applyDamping,
                                                  double* __restrict__ Fp, double* __restrict__ Fm, double* __restrict__ F0) {
    const int M = d.M, Nj = d.Nj;
    const size_t total = (size_t)d.members * M;
    for (size_t it = blockIdx.x * (size_t)blockDim.x + threadIdx.x; it < total; it += (size_t)gridDim.x * blockDim.x) {
        const int member = static_cast<int>(it / M);
        const int idx = static_cast<int>(it - (size_t)member * M);
        const int w = idx / Nj, j = idx - w * Nj;
        const long long o = member * d.memberStride;
        float2 ch[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) ch[q] = make_float2(0.f, 0.f);
        for (int c = 0; c < d.nt; ++c) {
            const int q = d.tq[c];
            ch[q] = vspec[((size_t)q * d.members + member) * M + idx];
        }
        const double maxSpeed = applyDamping ? __longlong_as_double((long long)maxSpeedBits[member]) : 0.0;
        mixed_project_store(d, idx, w, j, ch, elapsed, maxSpeed, applyDamping, Ap + o, Am + o, A0 + o, Fp + o, Fm + o, F0 + o);
    }
}

}  // namespace dev
}  // namespace wvgpu

// Register-resident warp FFTs and the y / x passes built on them.
//
// A line of N = 32*R complex values lives in one warp: lane t holds R values.
// An R-point DFT in registers, a twiddle by exp(+-2 pi i t k/N) and five
// shfl_xor butterfly stages across lanes give the N-point DFT with no shared
// memory and no block barrier.  Two orderings:
//   fft_P : input  x[t + 32 r] in register r of lane t (natural)
//           output X[k1 + R*brev5(t)] in register k1 of lane t (lane bit-reversed)
//   fft_Q : input in fft_P's output layout, output in natural layout
// (fft_Q with sign s is the transpose of fft_P with sign s; the DFT matrix is
// symmetric, so both compute the same transform.)  Inverse transforms of
// spectra use fft_P; forward transforms of physical rows produced by fft_P use
// fft_Q, so physical samples never leave registers.
#pragma once

#include "wv_kernels.cuh"

namespace wvgpu {
namespace dev {

__host__ __device__ constexpr int brev_bits(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
__host__ __device__ constexpr int ilog2c(int r) { return r <= 1 ? 0 : 1 + ilog2c(r >> 1); }

__device__ __forceinline__ float shfl_xor_v(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor_v(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ ff shfl_xor_v(ff v, int m) {
    return ff(__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m));
}

template <typename T>
__device__ __forceinline__ cx<T> shfl_xor_cx(cx<T> v, int m) {
    return mk<T>(shfl_xor_v(v.x, m), shfl_xor_v(v.y, m));
}

// Asynchronous global -> shared copies of one complex value (cp.async; 8-byte
// values through L1, 16-byte ones bypassing it), completed by wait_group.
template <typename T>
__device__ __forceinline__ void cp_async_cx(cx<T>* dst, const cx<T>* src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    if constexpr (sizeof(cx<T>) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// all but the most recent N committed groups of this thread have landed
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// s v + u for a lane sign s = +1 or -1 (the lane butterflies' one form); FP32 on
// one paired FFMA2 per value
template <typename T>
__device__ __forceinline__ cx<T> sign_add(T s, cx<T> v, cx<T> u) {
    if constexpr (std::is_same<T, float>::value) return __ffma2_rn(make_float2(s, s), v, u);
    else return mk<T>(s * v.x + u.x, s * v.y + u.y);
}

// multiply by exp(sigma * i pi / 2): -i (forward) or +i (inverse)
template <bool INV, typename T>
__device__ __forceinline__ cx<T> rot90(cx<T> b) { return INV ? mk<T>(-b.y, b.x) : mk<T>(b.y, -b.x); }

// One radix-2 layer of span LEN of the in-register DIT DFT, then the next
// (compile-time recursion, so that every register index is a constant: a
// runtime loop over the span left 16-point lines in local memory).
template <typename T, int R, bool INV, int LEN>
__device__ __forceinline__ void dft_layers(cx<T> (&v)[R], const cx<T>* tw, int N) {
    if constexpr (LEN <= R) {
#pragma unroll
        for (int i = 0; i < R; i += LEN) {
#pragma unroll
            for (int j = 0; j < LEN / 2; ++j) {
                const cx<T> a = v[i + j];
                cx<T> b = v[i + j + LEN / 2];
                if (j != 0) {
                    if (4 * j == LEN) b = rot90<INV, T>(b);
                    else b = cmul<T>(b, twid<T, INV>(tw, j * (N / LEN)));
                }
                v[i + j] = cadd<T>(a, b);
                v[i + j + LEN / 2] = csub<T>(a, b);
            }
        }
        dft_layers<T, R, INV, 2 * LEN>(v, tw, N);
    }
}

// 3-point DFT in place: t1 = v1 + v2, t2 = v0 - t1 / 2, t3 = i s (v1 - v2) with
// s = -sqrt(3)/2 (forward) or +sqrt(3)/2 (inverse); out = v0 + t1, t2 + t3, t2 - t3.
template <typename T, bool INV>
__device__ __forceinline__ void dft3(cx<T>& v0, cx<T>& v1, cx<T>& v2) {
    const T s3 = INV ? T(0.86602540378443864676) : T(-0.86602540378443864676);
    const cx<T> t1 = cadd<T>(v1, v2);
    const cx<T> t2 = mk<T>(v0.x - T(0.5) * t1.x, v0.y - T(0.5) * t1.y);
    const cx<T> dl = csub<T>(v1, v2);
    const cx<T> t3 = mk<T>(-(s3 * dl.y), s3 * dl.x);
    v0 = cadd<T>(v0, t1);
    v1 = cadd<T>(t2, t3);
    v2 = csub<T>(t2, t3);
}

// In-register R-point DFT, natural order in and out.  tw: N-entry table of
// exp(-2 pi i k/N) with R | N.  Radix 3 directly, 6 as 2 x 3 (the DFTs of the
// even and the odd samples, one twiddled radix-2 layer), other odd radices by
// the O(R^2) sum.
template <typename T, int R, bool INV>
__device__ __forceinline__ void small_dft(cx<T> (&v)[R], const cx<T>* tw, int N) {
    if constexpr (R == 1) {
        return;
    } else if constexpr (R == 3) {
        dft3<T, INV>(v[0], v[1], v[2]);
    } else if constexpr (R == 6) {
        cx<T> e0 = v[0], e1 = v[2], e2 = v[4], o0 = v[1], o1 = v[3], o2 = v[5];
        dft3<T, INV>(e0, e1, e2);
        dft3<T, INV>(o0, o1, o2);
        o1 = cmul<T>(o1, twid<T, INV>(tw, N / 6));
        o2 = cmul<T>(o2, twid<T, INV>(tw, 2 * (N / 6)));
        v[0] = cadd<T>(e0, o0); v[3] = csub<T>(e0, o0);
        v[1] = cadd<T>(e1, o1); v[4] = csub<T>(e1, o1);
        v[2] = cadd<T>(e2, o2); v[5] = csub<T>(e2, o2);
    } else if constexpr ((R & (R - 1)) == 0) {
        constexpr int LOG = ilog2c(R);
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int j = brev_bits(i, LOG);
            if (i < j) { const cx<T> t = v[i]; v[i] = v[j]; v[j] = t; }
        }
        dft_layers<T, R, INV, 2>(v, tw, N);
    } else {
        cx<T> out[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            cx<T> acc = v[0];
#pragma unroll
            for (int r = 1; r < R; ++r) acc = cadd<T>(acc, cmul<T>(v[r], twid<T, INV>(tw, ((r * k) % R) * (N / R))));
            out[k] = acc;
        }
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = out[k];
    }
}

// Paired FP32 in split form (ffs, wv_ff.cuh): the in-register DFTs.

template <int R, bool INV, int LEN>
__device__ __forceinline__ void s_dft_layers(ffs (&v)[R], const ff2* tw, int N) {
    if constexpr (LEN <= R) {
#pragma unroll
        for (int i = 0; i < R; i += LEN) {
#pragma unroll
            for (int j = 0; j < LEN / 2; ++j) {
                const ffs a = v[i + j];
                ffs b = v[i + j + LEN / 2];
                if (j != 0) {
                    if (4 * j == LEN) b = s_rot90<INV>(b);
                    else b = s_cmul(b, s_twiddle<INV>(tw, j * (N / LEN)));
                }
                v[i + j] = s_add(a, b);
                v[i + j + LEN / 2] = s_sub(a, b);
            }
        }
        s_dft_layers<R, INV, 2 * LEN>(v, tw, N);
    }
}

// dft3 in split form (the scalar form's operations per component)
template <bool INV>
__device__ __forceinline__ void s_dft3(ffs& v0, ffs& v1, ffs& v2) {
    const ff s3 = INV ? ff(0.86602540378443864676) : ff(-0.86602540378443864676);
    const ffs t1 = s_add(v1, v2);
    const ffs t2 = s_sub(v0, s_mul({f2(0.5f, 0.5f), f2(0.0f, 0.0f)}, t1));
    const ffs dl = s_sub(v1, v2);
    // (-(s3 dl.im), s3 dl.re)
    const ffs t3 = s_mul({f2(-s3.hi, s3.hi), f2(-s3.lo, s3.lo)}, {f2(dl.h.y, dl.h.x), f2(dl.l.y, dl.l.x)});
    v0 = s_add(v0, t1);
    v1 = s_add(t2, t3);
    v2 = s_sub(t2, t3);
}

template <int R, bool INV>
__device__ __forceinline__ void s_small_dft(ffs (&v)[R], const ff2* tw, int N) {
    if constexpr (R == 1) {
        return;
    } else if constexpr (R == 3) {
        s_dft3<INV>(v[0], v[1], v[2]);
    } else if constexpr (R == 6) {
        ffs e0 = v[0], e1 = v[2], e2 = v[4], o0 = v[1], o1 = v[3], o2 = v[5];
        s_dft3<INV>(e0, e1, e2);
        s_dft3<INV>(o0, o1, o2);
        o1 = s_cmul(o1, s_twiddle<INV>(tw, N / 6));
        o2 = s_cmul(o2, s_twiddle<INV>(tw, 2 * (N / 6)));
        v[0] = s_add(e0, o0); v[3] = s_sub(e0, o0);
        v[1] = s_add(e1, o1); v[4] = s_sub(e1, o1);
        v[2] = s_add(e2, o2); v[5] = s_sub(e2, o2);
    } else if constexpr ((R & (R - 1)) == 0) {
        constexpr int LOG = ilog2c(R);
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int j = brev_bits(i, LOG);
            if (i < j) { const ffs t = v[i]; v[i] = v[j]; v[j] = t; }
        }
        s_dft_layers<R, INV, 2>(v, tw, N);
    } else {
        ffs out[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            ffs acc = v[0];
#pragma unroll
            for (int r = 1; r < R; ++r) acc = s_add(acc, s_cmul(v[r], s_twiddle<INV>(tw, ((r * k) % R) * (N / R))));
            out[k] = acc;
        }
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = out[k];
    }
}

__device__ __forceinline__ ffs s_shfl_xor(ffs v, int m) {
    return {f2(__shfl_xor_sync(0xffffffffu, v.h.x, m), __shfl_xor_sync(0xffffffffu, v.h.y, m)),
            f2(__shfl_xor_sync(0xffffffffu, v.l.x, m), __shfl_xor_sync(0xffffffffu, v.l.y, m))};
}

// fft_P and fft_Q of paired FP32 values in split form (same data orders)
template <int R, bool INV>
__device__ __forceinline__ void s_fft_P(ff2 (&x)[R], const ff2* tw, int lane) {
    constexpr int N = 32 * R;
    ffs v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = to_split(x[r]);
    s_small_dft<R, INV>(v, tw, N);
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = s_cmul(v[k], s_twiddle<INV>(tw, lane * k));
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool bottom = (lane & h) != 0;
        const ffw w = bottom ? s_twiddle<INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : s_unit();
        const float sg = bottom ? -1.0f : 1.0f;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const ffs u = s_shfl_xor(v[r], h);
            v[r] = s_cmul(s_sign_add(sg, v[r], u), w);
        }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) x[r] = from_split(v[r]);
}

template <int R, bool INV>
__device__ __forceinline__ void s_fft_Q(ff2 (&x)[R], const ff2* tw, int lane) {
    constexpr int N = 32 * R;
    ffs v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = to_split(x[r]);
#pragma unroll
    for (int h = 1; h <= 16; h <<= 1) {
        const bool bottom = (lane & h) != 0;
        const ffw w = bottom ? s_twiddle<INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : s_unit();
        const float sg = bottom ? -1.0f : 1.0f;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const ffs m = s_cmul_left(w, v[r]);
            const ffs u = s_shfl_xor(m, h);
            v[r] = s_sign_add(sg, m, u);
        }
    }
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = s_cmul(v[k], s_twiddle<INV>(tw, lane * k));
    s_small_dft<R, INV>(v, tw, N);
#pragma unroll
    for (int r = 0; r < R; ++r) x[r] = from_split(v[r]);
}

// The lane butterflies take one form in every lane, with a per-lane sign and
// twiddle (1 in the top lanes, exactly), instead of evaluating the top and the
// bottom lane's expressions and selecting: 6 arithmetic instructions per value
// and stage instead of 10 (fft_P) or 14 (fft_Q), same roundings.
template <typename T, int R, bool INV>
__device__ __forceinline__ void fft_P(cx<T> (&v)[R], const cx<T>* tw, int lane) {
    if constexpr (std::is_same<T, ff>::value) {
        s_fft_P<R, INV>(v, tw, lane);
        return;
    }
    constexpr int N = 32 * R;
    small_dft<T, R, INV>(v, tw, N);
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = cmul<T>(v[k], twid<T, INV>(tw, lane * k));
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        // top lane: v + u;  bottom lane: (u - v) w   (u: the partner's value)
        const bool bottom = (lane & h) != 0;
        const cx<T> w = bottom ? twid<T, INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : mk<T>(T(1), T(0));
        const T sg = bottom ? T(-1) : T(1);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const cx<T> u = shfl_xor_cx<T>(v[r], h);
            v[r] = cmul<T>(sign_add<T>(sg, v[r], u), w);
        }
    }
}

template <typename T, int R, bool INV>
__device__ __forceinline__ void fft_Q(cx<T> (&v)[R], const cx<T>* tw, int lane) {
    if constexpr (std::is_same<T, ff>::value) {
        s_fft_Q<R, INV>(v, tw, lane);
        return;
    }
    constexpr int N = 32 * R;
#pragma unroll
    for (int h = 1; h <= 16; h <<= 1) {
        // top lane: v + w u;  bottom lane: u - w v   (u: the partner's value): the
        // bottom lane forms w v before the exchange, the top lane's factor is 1
        const bool bottom = (lane & h) != 0;
        const cx<T> w = bottom ? twid<T, INV>(tw, (lane & (h - 1)) * (N / (2 * h))) : mk<T>(T(1), T(0));
        const T sg = bottom ? T(-1) : T(1);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const cx<T> m = cmul<T>(w, v[r]);
            const cx<T> u = shfl_xor_cx<T>(m, h);
            v[r] = sign_add<T>(sg, m, u);
        }
    }
#pragma unroll
    for (int k = 1; k < R; ++k) v[k] = cmul<T>(v[k], twid<T, INV>(tw, lane * k));
    small_dft<T, R, INV>(v, tw, N);
}

// Index of register k1 of lane t in fft_P's output.
template <int R>
__device__ __forceinline__ int p_index(int k1, int lane) { return k1 + R * brev_bits(lane, 5); }

constexpr int kWG = 8;  // kx columns (y pass) or rows (x pass) per CTA: one per warp

// Slot of element (row y, column c) of an [N][kWG] transpose tile, N = 32*R:
// columns XOR-swizzled by bits of (y>>1) ^ (y/R >> 2).  A warp storing the
// rows k1 + R*brev5(lane) of one column (fft_P's output) meets 2-way bank
// conflicts at most; loading the rows lane + 32r of one column, or sweeping
// the tile row-major, meets none (checked for R = 1, 2, 3, 4, 6, 8, 16).
template <int R>
__device__ __forceinline__ int tile_at(int y, int c) {
    return y * kWG + (c ^ (((y >> 1) ^ ((y / R) >> 2)) & (kWG - 1)));
}

// ---------------------------------------------------------------------------
// y inverse: CTA = (8 kx columns, plane z, output channel); warp = one column.

template <typename T, int R>
__global__ void __launch_bounds__(256) k_yinv_w(DescDev d, YInvMap map, const cx<T>* __restrict__ zspec,
                                               cx<T>* __restrict__ yspec) {
    constexpr int N = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);   // [N]
    cx<T>* tile = tw + N;                              // [N][kWG]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int kx0 = blockIdx.x * kWG, z = blockIdx.y, oc = blockIdx.z;
    const int KX = d.kxColumns, P = d.positions;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = twg[i];
    __syncthreads();
    const int kx = kx0 + warp;
    if (kx < KX) {
        const cx<T>* in = zspec + ((size_t)map.src[oc] * d.zTotal + z) * P;
        const int* ym = d.ymap + (size_t)kx * N;
        const bool mulL = map.mulL[oc] != 0;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int y = lane + 32 * r;
            const int pos = ym[y];
            cx<T> val = pos >= 0 ? in[pos] : mk<T>(T(0), T(0));
            if (mulL) {
                const T l = row_l<T>(d)[y];
                val = mk<T>(-l * val.y, l * val.x);
            }
            v[r] = val;
        }
        fft_P<T, R, true>(v, tw, lane);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) tile[tile_at<R>(p_index<R>(k1, lane), warp)] = v[k1];
    }
    __syncthreads();
    const int g = min(kWG, KX - kx0);
    cx<T>* out = yspec + (((size_t)z * map.nOut + oc) * N) * KX + kx0;
    for (int i = threadIdx.x; i < N * kWG; i += blockDim.x) {
        const int y = i / kWG, gi = i - y * kWG;
        if (gi < g) out[(size_t)y * KX + gi] = tile[tile_at<R>(y, gi)];
    }
}

// y forward: CTA = (8 kx columns, plane z, channel); gathered to active rows.
template <typename T, int R>
__global__ void __launch_bounds__(256) k_yfwd_w(DescDev d, const cx<T>* __restrict__ pspec, int nch,
                                               cx<T>* __restrict__ fspec) {
    constexpr int N = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* tile = tw + N;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int kx0 = blockIdx.x * kWG, z = blockIdx.y, c = blockIdx.z;
    const int KX = d.kxColumns, P = d.positions;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = twg[i];
    const int g = min(kWG, KX - kx0);
    const cx<T>* in = pspec + (((size_t)z * nch + c) * N) * KX + kx0;
    for (int i = threadIdx.x; i < N * kWG; i += blockDim.x) {
        const int y = i / kWG, gi = i - y * kWG;
        tile[tile_at<R>(y, gi)] = gi < g ? in[(size_t)y * KX + gi] : mk<T>(T(0), T(0));
    }
    __syncthreads();
    const int kx = kx0 + warp;
    if (kx >= KX) return;
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = tile[tile_at<R>(lane + 32 * r, warp)];
    fft_P<T, R, false>(v, tw, lane);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) tile[tile_at<R>(p_index<R>(k1, lane), warp)] = v[k1];
    __syncwarp();
    cx<T>* out = fspec + ((size_t)c * d.zTotal + z) * P;
    const int pBeg = d.colStart[kx], pEnd = d.colStart[kx + 1];
    for (int p = pBeg + lane; p < pEnd; p += 32) out[p] = tile[tile_at<R>(d.posKy[p], warp)];
}

// ---------------------------------------------------------------------------
// x pass: one warp per (y, z) row, 8 rows per CTA.  Real rows of Nx = 64*R
// samples are complex lines of L = 32*R (even/odd sample split); physical
// samples 2n, 2n+1 with n = k1 + R*brev5(lane) stay in registers.

template <typename T, int R>
__device__ __forceinline__ void c2r_row(const DescDev& d, const cx<T>* h, bool useK, const cx<T>* twL, const cx<T>* twN,
                                        int lane, cx<T> (&v)[R]) {
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = c2r_line_entry<T>(d, h, lane + 32 * q, useK, twN);
    fft_P<T, R, true>(v, twL, lane);
}

// Row i of the x pass (0: U, 1: V, 2: W, then (q_x, q_y, q_z) per target) ->
// its input channel of the y spectra; q_x is channel q times i k.
__device__ __forceinline__ int xrow_channel(const DescDev& d, int i) {
    if (i < 3) return i;
    const int t = (i - 3) / 3, kind = (i - 3) - 3 * t;
    return kind == 0 ? d.tq[t] : (kind == 1 ? 4 + t : 4 + d.nt + t);
}

// Shared-memory stage of one warp's channel rows: two buffers of KX values,
// padded to an even count (16-byte aligned buffers).
__host__ __device__ inline int xstage_len(int KX) { return (KX + 1) & ~1; }
// ... of the x-pass adjoint: a spectrum row (KX values) or a kept real row (L values)
__host__ __device__ inline int xadj_stage_len(int L, int KX) { return L > xstage_len(KX) ? L : xstage_len(KX); }

// physOut, when given, receives the real rows as complex pairs in register
// order: [z][nReal][y][L], entry k*32 + lane = register k of lane `lane`.
// advOut / advIn: the advecting (u, v, w) as doubles [3][z][y][Nx], written out
// or taken in place of the reconstructed ones (sample pair 2n, 2n+1 of the row
// sits in register k of lane l with n = k + R brev5(l)).
// CTAs per SM the x pass is compiled for: FP32 rows of up to 4 registers per
// lane fit 64 registers without spilling (4 CTAs, 32 warps per SM); longer rows
// take 2 CTAs (their register tiles would spill at 3)
template <typename T, int R>
__host__ __device__ constexpr int xflux_min_blocks() { return sizeof(T) == 4 && R <= 4 ? 4 : 2; }

template <typename T, int R>
__global__ void __launch_bounds__(256, xflux_min_blocks<T, R>()) k_xflux_w(DescDev d, const cx<T>* __restrict__ yspec, cx<T>* __restrict__ pspec,
                                                unsigned long long* __restrict__ maxSpeedBits, cx<T>* __restrict__ physOut,
                                                double* __restrict__ advOut, const double* __restrict__ advIn) {
    constexpr int L = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double warpMax[kWG];
    __shared__ int warpsDone;
    const int Ny = d.Ny, KX = d.kxColumns, nt = d.nt;
    const int nIn = 4 + 2 * nt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int z = blockIdx.y;
    const int y = blockIdx.x * kWG + warp;
    cx<T>* twL = reinterpret_cast<cx<T>*>(smem_raw);   // [L]
    cx<T>* twN = twL + L;                               // [2L]
    cx<T>* line = twN + 2 * L + warp * L;               // per warp: [L]
    const int KXs = xstage_len(KX);
    cx<T>* stage = twN + 2 * L + kWG * L + warp * 2 * KXs;  // per warp: [2][KXs]
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) twL[i] = twg[i];
    for (int i = threadIdx.x; i < 2 * L; i += blockDim.x) twN[i] = twgN[i];
    if (threadIdx.x == 0) warpsDone = 0;
    __syncthreads();
    if (y >= Ny) return;
    // spectra of this row: channel c at row + c*Ny*KX.  Each channel row is
    // copied to the warp's stage asynchronously two rows ahead of its use, so
    // its global-memory latency overlaps the FFTs of the rows before it.
    const cx<T>* row = yspec + (((size_t)z * nIn) * Ny + y) * KX;
    const size_t cstride = (size_t)Ny * KX;
    const int nReal = 3 + 3 * nt;
    auto fetch = [&](int i) {
        if (i < nReal) {
            const cx<T>* src = row + xrow_channel(d, i) * cstride;
            cx<T>* dst = stage + (i & 1) * KXs;
            for (int k = lane; k < KX; k += 32) cp_async_cx<T>(dst + k, src + k);
        }
        cp_async_commit();  // an empty group past the last row keeps the count uniform
    };
    // row i from its stage buffer; the buffer is refilled with row i + 2 after every lane has read it
    auto build = [&](int i, bool useK, cx<T> (&out)[R]) {
        cp_async_wait<1>();
        __syncwarp();
        c2r_row<T, R>(d, stage + (i & 1) * KXs, useK, twL, twN, lane, out);
        __syncwarp();
        fetch(i + 2);
    };
    fetch(0);
    fetch(1);
    cx<T> U[R], V[R], W[R], v[R], S[R];
    build(0, false, U);
    build(1, false, V);
    build(2, false, W);
    auto keep = [&](int r, const cx<T> (&x)[R]) {
        cx<T>* o = physOut + (((size_t)z * nReal + r) * Ny + y) * L + lane;
#pragma unroll
        for (int k = 0; k < R; ++k) o[32 * k] = x[k];
    };
    if (advIn || advOut) {
        const size_t R3 = (size_t)(2 * L) * Ny * d.Nz;
        const size_t rowOff = ((size_t)z * Ny + y) * (2 * L);
        cx<T>* vel[3] = {U, V, W};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const size_t g = (size_t)c * R3 + rowOff + 2 * (size_t)p_index<R>(k, lane);
                if (advIn) {
                    const double2 a = *reinterpret_cast<const double2*>(advIn + g);
                    vel[c][k] = mk<T>(T(a.x), T(a.y));
                } else {
                    *reinterpret_cast<double2*>(advOut + g) = make_double2(double(vel[c][k].x), double(vel[c][k].y));
                }
            }
        }
    }
    if (physOut) { keep(0, U); keep(1, V); keep(2, W); }
    // max |u_h| only when a consumer asked for it (max of u^2 + v^2, one sqrt at the end)
    const bool wantSpeed = maxSpeedBits != nullptr;
    double vmax2 = 0.0;
    if (wantSpeed) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            vmax2 = fmax(vmax2, double(U[k].x) * double(U[k].x) + double(V[k].x) * double(V[k].x));
            vmax2 = fmax(vmax2, double(U[k].y) * double(U[k].y) + double(V[k].y) * double(V[k].y));
        }
    }
#pragma unroll 1
    for (int t = 0; t < nt; ++t) {
        // S_q = -(u q_x + v q_y + w q_z), accumulated in that order
#pragma unroll 1
        for (int kind = 0; kind < 3; ++kind) {
            build(3 + 3 * t + kind, kind == 0, v);
            if (physOut) keep(3 + 3 * t + kind, v);
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const cx<T> m = kind == 0 ? U[k] : (kind == 1 ? V[k] : W[k]);
                const cx<T> p = mk<T>(m.x * v[k].x, m.y * v[k].y);
                S[k] = kind == 0 ? p : mk<T>(S[k].x + p.x, S[k].y + p.y);
            }
        }
#pragma unroll
        for (int k = 0; k < R; ++k) S[k] = mk<T>(-S[k].x, -S[k].y);
        fft_Q<T, R, false>(S, twL, lane);
#pragma unroll
        for (int qq = 0; qq < R; ++qq) line[lane + 32 * qq] = S[qq];
        __syncwarp();
        cx<T>* out = pspec + (((size_t)z * nt + t) * Ny + y) * KX;
        for (int k = lane; k < KX; k += 32) out[k] = r2c_value<T>(d, line, k, twN);
        __syncwarp();
    }
    if (!wantSpeed) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax2 = fmax(vmax2, __shfl_xor_sync(0xffffffffu, vmax2, o));
    // one atomic per CTA: the rows of this CTA reduce through shared memory
    if (lane == 0) {
        warpMax[warp] = vmax2;
        __threadfence_block();
        const int rows = min(kWG, Ny - (int)blockIdx.x * kWG);
        if (atomicAdd(&warpsDone, 1) == rows - 1) {
            double m = 0.0;
            for (int i = 0; i < rows; ++i) m = fmax(m, warpMax[i]);
            atomicMax(maxSpeedBits + z / d.Nz, (unsigned long long)__double_as_longlong(sqrt(m)));
        }
    }
}

// ---------------------------------------------------------------------------
// x pass adjoint (transpose of k_xflux_w), one warp per (y, z) row, 8 rows per
// CTA.  Forward rows U, V, W and the gradients of the value rows stay in
// registers; per target: adjoint row s (c2r with interior kx at weight 1/2,
// i.e. 0.5 c2r(h) + 0.5 Re h[0]), the forward rows q_x, q_y, q_z, and the
// gradient rows -s U, -s V, -s W through r2c with interior kx doubled.  The
// -i k x-derivative gradient is parked per warp in shared memory and added to
// its value channel at the end.  Output in the forward y-spectrum layout.

template <typename T, int R>
__device__ __forceinline__ void r2c_row_to_line(cx<T> (&g)[R], const cx<T>* twL, cx<T>* line, int lane) {
    fft_Q<T, R, false>(g, twL, lane);
#pragma unroll
    for (int qq = 0; qq < R; ++qq) line[lane + 32 * qq] = g[qq];
    __syncwarp();
}

// physIn, when given, holds the forward real rows as k_xflux_w keeps them;
// otherwise they are recomputed from yspec.
template <typename T, int R>
__global__ void __launch_bounds__(256, 2) k_xadj_w(DescDev d, const cx<T>* __restrict__ yspec, const cx<T>* __restrict__ yadj,
                                                cx<T>* __restrict__ yout, const cx<T>* __restrict__ physIn) {
    constexpr int L = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, KX = d.kxColumns, nt = d.nt;
    const int nIn = 4 + 2 * nt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int z = blockIdx.y;
    const int y = blockIdx.x * kWG + warp;
    cx<T>* twL = reinterpret_cast<cx<T>*>(smem_raw);   // [L]
    cx<T>* twN = twL + L;                               // [2L]
    cx<T>* line = twN + 2 * L + warp * (L + 4 * KX);    // per warp: [L] line, [4][KX] x-derivative parts
    cx<T>* xpart = line + L;
    const int SL = xadj_stage_len(L, KX);
    cx<T>* stage = twN + 2 * L + kWG * (L + 4 * KX) + warp * 2 * SL;  // per warp: [2][SL]
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) twL[i] = twg[i];
    for (int i = threadIdx.x; i < 2 * L; i += blockDim.x) twN[i] = twgN[i];
    __syncthreads();
    if (y >= Ny) return;
    const size_t cstride = (size_t)Ny * KX;
    const cx<T>* row = yspec + (((size_t)z * nIn) * Ny + y) * KX;
    const cx<T>* arow = yadj + (((size_t)z * nt) * Ny + y) * KX;
    cx<T>* orow = yout + (((size_t)z * nIn) * Ny + y) * KX;
    for (int i = lane; i < 4 * KX; i += 32) xpart[i] = mk<T>(T(0), T(0));
    __syncwarp();
    cx<T> U[R], V[R], W[R], gu[R], gv[R], gw[R], sb[R], v[R], g[R];
    const int nReal = 3 + 3 * nt;
    // Inputs in the order of use: forward rows 0..2 (U, V, W), then per target
    // its adjoint row and its forward rows q_x, q_y, q_z.  Each is copied to the
    // warp's stage asynchronously two inputs ahead of its use: a forward row
    // kept by the forward pass (L values in register order) or a spectrum row
    // (KX values) for a c2r.
    const int nItems = 3 + 4 * nt;
    auto fwdIndex = [&](int i) { return i < 3 ? i : 3 + 3 * ((i - 3) / 4) + ((i - 3) % 4) - 1; };
    auto fetch = [&](int i) {
        if (i < nItems) {
            cx<T>* dst = stage + (i & 1) * SL;
            const bool adjRow = i >= 3 && (i - 3) % 4 == 0;
            if (adjRow) {
                const cx<T>* src = arow + ((i - 3) / 4) * cstride;
                for (int k = lane; k < KX; k += 32) cp_async_cx<T>(dst + k, src + k);
            } else if (physIn) {
                const cx<T>* src = physIn + (((size_t)z * nReal + fwdIndex(i)) * Ny + y) * L;
#pragma unroll
                for (int k = 0; k < R; ++k) cp_async_cx<T>(dst + lane + 32 * k, src + lane + 32 * k);
            } else {
                const cx<T>* src = row + xrow_channel(d, fwdIndex(i)) * cstride;
                for (int k = lane; k < KX; k += 32) cp_async_cx<T>(dst + k, src + k);
            }
        }
        cp_async_commit();  // an empty group past the last input keeps the count uniform
    };
    auto take = [&](int i) -> const cx<T>* {
        cp_async_wait<1>();
        __syncwarp();
        return stage + (i & 1) * SL;
    };
    auto release = [&](int i) {  // every lane is done with input i's buffer
        __syncwarp();
        fetch(i + 2);
    };
    // forward real row of input i (register order)
    auto fwdRow = [&](int i, bool useK, cx<T> (&x)[R]) {
        const cx<T>* b = take(i);
        if (physIn) {
#pragma unroll
            for (int k = 0; k < R; ++k) x[k] = b[lane + 32 * k];
        } else {
            c2r_row<T, R>(d, b, useK, twL, twN, lane, x);
        }
        release(i);
    };
    fetch(0);
    fetch(1);
    fwdRow(0, false, U);
    fwdRow(1, false, V);
    fwdRow(2, false, W);
#pragma unroll
    for (int k = 0; k < R; ++k) { gu[k] = mk<T>(T(0), T(0)); gv[k] = gu[k]; gw[k] = gu[k]; }
    // half-spectrum r2c of g into output channel ch (or the x-derivative part of value channel q)
    auto put = [&](cx<T> (&gr)[R], int ch, int xq) {
        r2c_row_to_line<T, R>(gr, twL, line, lane);
        for (int k = lane; k < KX; k += 32) {
            cx<T> val = r2c_value<T>(d, line, k, twN);
            if (k > 0) val = mk<T>(T(2) * val.x, T(2) * val.y);
            if (xq >= 0) {
                const T kk = row_k<T>(d)[k];
                xpart[xq * KX + k] = mk<T>(kk * val.y, -kk * val.x);   // (i k)^* = -i k
            } else {
                orow[(size_t)ch * cstride + k] = val;
            }
        }
        __syncwarp();
    };
#pragma unroll 1
    for (int t = 0; t < nt; ++t) {
        const int q = d.tq[t];
        const int ia = 3 + 4 * t;  // input index of the adjoint row
        {
            const cx<T>* b = take(ia);
            c2r_row<T, R>(d, b, false, twL, twN, lane, sb);
            const T h0 = b[0].x;  // imaginary part dropped by c2r
#pragma unroll
            for (int k = 0; k < R; ++k) sb[k] = mk<T>(T(0.5) * sb[k].x + T(0.5) * h0, T(0.5) * sb[k].y + T(0.5) * h0);
            release(ia);
        }
#pragma unroll 1
        for (int kind = 0; kind < 3; ++kind) {
            const int ch = kind == 0 ? q : (kind == 1 ? 4 + t : 4 + nt + t);
            fwdRow(ia + 1 + kind, kind == 0, v);
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const cx<T> p = mk<T>(sb[k].x * v[k].x, sb[k].y * v[k].y);
                if (kind == 0) gu[k] = mk<T>(gu[k].x - p.x, gu[k].y - p.y);
                else if (kind == 1) gv[k] = mk<T>(gv[k].x - p.x, gv[k].y - p.y);
                else gw[k] = mk<T>(gw[k].x - p.x, gw[k].y - p.y);
                const cx<T> m = kind == 0 ? U[k] : (kind == 1 ? V[k] : W[k]);
                g[k] = mk<T>(-sb[k].x * m.x, -sb[k].y * m.y);
            }
            // gradient of q_x (x-derivative of channel q), q_y (channel 4+t), q_z (channel 4+nt+t)
            put(g, ch, kind == 0 ? q : -1);
        }
    }
    // value channels: r2c of the accumulated gradients plus the x-derivative parts
    for (int c = 0; c < 4; ++c) {
        if (c < 3) {
            if (c == 0) r2c_row_to_line<T, R>(gu, twL, line, lane);
            else if (c == 1) r2c_row_to_line<T, R>(gv, twL, line, lane);
            else r2c_row_to_line<T, R>(gw, twL, line, lane);
        }
        for (int k = lane; k < KX; k += 32) {
            cx<T> val = mk<T>(T(0), T(0));
            if (c < 3) {
                val = r2c_value<T>(d, line, k, twN);
                if (k > 0) val = mk<T>(T(2) * val.x, T(2) * val.y);
            }
            const cx<T> xp = xpart[c * KX + k];
            orow[(size_t)c * cstride + k] = mk<T>(val.x + xp.x, val.y + xp.y);
        }
        __syncwarp();
    }
}

// y forward of the x-pass adjoint's output, y-derivative channels folded onto
// their source channel (see k_yfwd_pair); one warp per kx column.
template <typename T, int R>
__global__ void __launch_bounds__(256) k_yfwd_pair_w(DescDev d, YFwdPairMap map, const cx<T>* __restrict__ pspec, int nIn,
                                                    cx<T>* __restrict__ fspec) {
    constexpr int N = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* tileA = tw + N;
    cx<T>* tileB = tileA + N * kWG;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int kx0 = blockIdx.x * kWG, z = blockIdx.y, c = blockIdx.z;
    const int KX = d.kxColumns, P = d.positions;
    const int a = map.srcA[c], b = map.srcB[c];
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = twg[i];
    const int g = min(kWG, KX - kx0);
    auto fill = [&](int ch, cx<T>* tile) {
        const cx<T>* in = pspec + (((size_t)z * nIn + ch) * N) * KX + kx0;
        for (int i = threadIdx.x; i < N * kWG; i += blockDim.x) {
            const int y = i / kWG, gi = i - y * kWG;
            tile[tile_at<R>(y, gi)] = gi < g ? in[(size_t)y * KX + gi] : mk<T>(T(0), T(0));
        }
    };
    fill(a, tileA);
    if (b >= 0) fill(b, tileB);
    __syncthreads();
    const int kx = kx0 + warp;
    if (kx >= KX) return;
    auto transform = [&](cx<T>* tile) {
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = tile[tile_at<R>(lane + 32 * r, warp)];
        fft_P<T, R, false>(v, tw, lane);
        __syncwarp();
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) tile[tile_at<R>(p_index<R>(k1, lane), warp)] = v[k1];
        __syncwarp();
    };
    transform(tileA);
    if (b >= 0) transform(tileB);
    cx<T>* out = fspec + ((size_t)c * d.zTotal + z) * P;
    const T* rl = row_l<T>(d);
    const int pBeg = d.colStart[kx], pEnd = d.colStart[kx + 1];
    for (int p = pBeg + lane; p < pEnd; p += 32) {
        const int ky = d.posKy[p];
        cx<T> v = tileA[tile_at<R>(ky, warp)];
        if (b >= 0) {
            const cx<T> w = tileB[tile_at<R>(ky, warp)];
            const T l = rl[ky];
            v = mk<T>(v.x + l * w.y, v.y - l * w.x);
        }
        out[p] = v;
    }
}

// inverse fields: c2r of nch channels to fields[ch][z][y][x]
template <typename T, int R>
__global__ void __launch_bounds__(256) k_xc2r_fields_w(DescDev d, const cx<T>* __restrict__ yspec, int nch,
                                                      double* __restrict__ fields) {
    constexpr int L = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, Nz = d.Nz, KX = d.kxColumns, Nx = 2 * L;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int z = blockIdx.y;
    const int y = blockIdx.x * kWG + warp;
    cx<T>* twL = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* twN = twL + L;
    cx<T>* spec = twN + 2 * L + warp * (nch * KX + L);
    cx<T>* line = spec + nch * KX;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) twL[i] = twg[i];
    for (int i = threadIdx.x; i < 2 * L; i += blockDim.x) twN[i] = twgN[i];
    __syncthreads();
    if (y >= Ny) return;
    for (int i = lane; i < nch * KX; i += 32) {
        const int c = i / KX, k = i - c * KX;
        spec[i] = yspec[(((size_t)z * nch + c) * Ny + y) * KX + k];
    }
    __syncwarp();
    const size_t R3 = (size_t)Nx * Ny * Nz;
    for (int c = 0; c < nch; ++c) {
        cx<T> v[R];
        c2r_row<T, R>(d, spec + c * KX, ((d.c2rUseK >> c) & 1) != 0, twL, twN, lane, v);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) line[p_index<R>(k1, lane)] = v[k1];
        __syncwarp();
        double* out = fields + (size_t)c * R3 + ((size_t)z * Ny + y) * Nx;
        const T* samples = reinterpret_cast<const T*>(line);
        for (int x = lane; x < Nx; x += 32) out[x] = double(samples[x]);
        __syncwarp();
    }
}

// forward fields: r2c of field rows -> pspec[z][ch][y][kx]
template <typename T, int R>
__global__ void __launch_bounds__(256) k_xr2c_fields_w(DescDev d, const double* __restrict__ fields, int nch,
                                                      cx<T>* __restrict__ pspec) {
    constexpr int L = 32 * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, Nz = d.Nz, KX = d.kxColumns, Nx = 2 * L;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int z = blockIdx.y;
    const int y = blockIdx.x * kWG + warp;
    cx<T>* twL = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* twN = twL + L;
    cx<T>* line = twN + 2 * L + warp * L;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) twL[i] = twg[i];
    for (int i = threadIdx.x; i < 2 * L; i += blockDim.x) twN[i] = twgN[i];
    __syncthreads();
    if (y >= Ny) return;
    const size_t R3 = (size_t)Nx * Ny * Nz;
    for (int c = 0; c < nch; ++c) {
        const double* row = fields + (size_t)c * R3 + ((size_t)z * Ny + y) * Nx;
        T* samples = reinterpret_cast<T*>(line);
        for (int x = lane; x < Nx; x += 32) samples[x] = T(row[x]);
        __syncwarp();
        cx<T> v[R];
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) v[k1] = line[p_index<R>(k1, lane)];
        __syncwarp();
        fft_Q<T, R, false>(v, twL, lane);
#pragma unroll
        for (int qq = 0; qq < R; ++qq) line[lane + 32 * qq] = v[qq];
        __syncwarp();
        cx<T>* out = pspec + (((size_t)z * nch + c) * Ny + y) * KX;
        for (int k = lane; k < KX; k += 32) out[k] = r2c_value<T>(d, line, k, twN);
        __syncwarp();
    }
}

}  // namespace dev
}  // namespace wvgpu

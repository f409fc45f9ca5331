// F-grid scalar advection (advectFGridScalar, kernel.cpp:1032-1138) on the
// full half spectrum: every (kx, ky) row is a position (pos = kx Ny + ky), the
// y kernels run with kx_columns = NxHalf, and the vertical derivative of each
// column is one dense Nz x Nz contraction (forward DCT-I with its
// normalization, times -m_j on the interior modes, normalizeInverseDST and
// DST-I on the interior points, folded on the host into D).
#pragma once

#include "wv_kernels.cuh"

namespace wvgpu {
namespace dev {

constexpr int kScalarCols = 32;  // positions per CTA of k_scalar_derivs

// in: channel spectra [z][pos] of the scalar after the y forward FFT (unscaled).
// out: [3][z][pos] = i k v, i l v, D v with v = hs * in; self-conjugate rows real.
// flags[pos]: bit 0 self-conjugate row.
template <typename T>
__global__ void __launch_bounds__(256) k_scalar_derivs(DescDev d, const cx<T>* __restrict__ in, const T* __restrict__ D,
                                                      const unsigned char* __restrict__ flags, double hs,
                                                      cx<T>* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* v = reinterpret_cast<cx<T>*>(smem_raw);  // [Nz][kScalarCols]
    const int P = d.positions, Nz = d.Nz, Ny = d.Ny;
    const int pos0 = blockIdx.x * kScalarCols;
    const int np = min(kScalarCols, P - pos0);
    const T s = T(hs);
    for (int i = threadIdx.x; i < Nz * kScalarCols; i += blockDim.x) {
        const int z = i / kScalarCols, pp = i - z * kScalarCols;
        cx<T> a = mk<T>(T(0), T(0));
        if (pp < np) { a = in[(size_t)z * P + pos0 + pp]; a = mk<T>(a.x * s, a.y * s); }
        v[i] = a;
    }
    __syncthreads();
    const T* rk = row_k<T>(d);
    const T* rl = row_l<T>(d);
    for (int i = threadIdx.x; i < Nz * kScalarCols; i += blockDim.x) {
        const int z = i / kScalarCols, pp = i - z * kScalarCols;
        if (pp >= np) continue;
        const int pos = pos0 + pp;
        const int kx = pos / Ny, ky = pos - kx * Ny;
        const cx<T> val = v[i];
        const T k = rk[kx], l = rl[ky];
        cx<T> cxv = mk<T>(-k * val.y, k * val.x);
        cx<T> cyv = mk<T>(-l * val.y, l * val.x);
        T re = T(0), im = T(0);
        const T* Dz = D + (size_t)z * Nz;
        for (int zz = 0; zz < Nz; ++zz) {
            const cx<T> w = v[zz * kScalarCols + pp];
            re += Dz[zz] * w.x;
            im += Dz[zz] * w.y;
        }
        cx<T> czv = mk<T>(re, im);
        if (flags[pos] & 1) { cxv.y = T(0); cyv.y = T(0); czv.y = T(0); }
        out[(size_t)(0 * Nz + z) * P + pos] = cxv;
        out[(size_t)(1 * Nz + z) * P + pos] = cyv;
        out[(size_t)(2 * Nz + z) * P + pos] = czv;
    }
}

// Antialias filter in place on [z][pos]: rows with flag bit 1 keep hs * v, others 0.
template <typename T>
__global__ void k_scalar_mask(DescDev d, cx<T>* __restrict__ v, const unsigned char* __restrict__ flags, double hs) {
    const size_t n = (size_t)d.Nz * d.positions;
    const T s = T(hs);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int pos = static_cast<int>(i % d.positions);
        const cx<T> a = v[i];
        v[i] = (flags[pos] & 2) ? mk<T>(a.x * s, a.y * s) : mk<T>(T(0), T(0));
    }
}

// rhs = -(u dx + v dy + w dz), all [R] doubles; grad = (dx, dy, dz), adv = (u, v, w).
__global__ void k_scalar_rhs(const double* __restrict__ grad, const double* __restrict__ adv, size_t R, double* __restrict__ rhs) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < R; i += (size_t)gridDim.x * blockDim.x)
        rhs[i] = -(adv[i] * grad[i] + adv[R + i] * grad[R + i] + adv[2 * R + i] * grad[2 * R + i]);
}

}  // namespace dev
}  // namespace wvgpu

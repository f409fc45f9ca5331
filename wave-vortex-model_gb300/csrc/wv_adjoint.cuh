// Adjoint (vector-Jacobian product) kernels of the nonlinear flux and of the
// inverse transform.  No counterpart in the reference.  Inner product on complex
// arrays: <a, b> = Re sum conj(a) b; every stage below is the transpose of the
// forward stage of the same name in wv_kernels.cuh:
//   k_vfwd_adj : projection and phase (transposed), forward vertical matrices
//                transposed -> per-target profiles at the stored rows
//   (y inverse of those profiles: the forward y kernels, unchanged)
//   k_xadj     : c2r of the forward rows and of the adjoint rows (interior kx
//                halved: adjoint of r2c), product adjoint, r2c of the gradient
//                rows (interior kx doubled: adjoint of c2r), -i k for the
//                x-derivative rows; written in the forward y-spectrum layout
//   (y forward of those: the forward y kernels, unchanged)
//   k_vinv_adj : -i l for the y-derivative channels, completion rows folded back
//                conjugated, inverse vertical matrices transposed, field
//                assembly and phase transposed -> (Ap, Am, A0) cotangents
#pragma once

#include "wv_kernels.cuh"

namespace wvgpu {
namespace dev {

// ---------------------------------------------------------------------------
// Cotangents of the transformed target channels (canonical frame, index t of
// the targets) of one (mode, j): the projection and phase of k_vfwd transposed.
template <typename T>
__device__ __forceinline__ void vfwd_adj_values(const DescDev& d, const double* __restrict__ Fpb,
                                                const double* __restrict__ Fmb, const double* __restrict__ F0b,
                                                double elapsed, int w, int j, cx<T> (&vt)[4]) {
    const int Nj = d.Nj, nt = d.nt;
    const int idx = j + Nj * w;
    if constexpr (sizeof(T) == 4) {
        // MIXED: transpose of the folded FP32 projection of k_vfwd, FP32 phase
        // after FP64 angle reduction
        const double ang = d.omega[idx] * elapsed;
        const double red = ang - 6.283185307179586476925 * rint(ang * 0.15915494309189533577);
        float sn, cs;
        sincosf(float(red), &sn, &cs);
        const float2 fpb = make_float2(float(Fpb[2 * idx]), float(Fpb[2 * idx + 1]));
        const float2 fmb = make_float2(float(Fmb[2 * idx]), float(Fmb[2 * idx + 1]));
        const float2 a0b = make_float2(float(F0b[2 * idx]), float(F0b[2 * idx + 1]));
        const float2 cpb = make_float2(fpb.x * cs - fpb.y * sn, fpb.x * sn + fpb.y * cs);  // Fp_bar * p
        const float2 cmb = make_float2(fmb.x * cs + fmb.y * sn, fmb.y * cs - fmb.x * sn);  // Fm_bar * conj(p)
        float2 ch[4];
        if (w == 0) {
            const float sc = float(d.inertialScale[j]);
            const float2 tot = make_float2(cpb.x + cmb.x, cpb.y - cmb.y);  // cp_bar + conj(cm_bar)
            ch[0] = make_float2(sc * tot.x, sc * tot.y);
            ch[1] = make_float2(-sc * tot.y, sc * tot.x);
            ch[2] = make_float2(0.f, 0.f);
            const float dn = d.fProj[12 * (size_t)idx + 8];
            ch[3] = make_float2(dn * a0b.x, dn * a0b.y);
        } else {
            const float4* pj = reinterpret_cast<const float4*>(d.fProj + 12 * (size_t)idx);
            const float4 p0 = pj[0], p1 = pj[1], p2 = pj[2];
            const float2 wb = make_float2(cpb.x + cmb.x, cpb.y + cmb.y);
            const float2 bb = make_float2(cpb.x - cmb.x, cpb.y - cmb.y);
            const float2 f0b = make_float2(a0b.x - p2.z * bb.x, a0b.y - p2.z * bb.y);
            // conj(C) * wave_bar - i D * f0_bar
            ch[0] = make_float2(p0.x * wb.x + p0.y * wb.y + p1.z * f0b.y, p0.x * wb.y - p0.y * wb.x - p1.z * f0b.x);
            ch[1] = make_float2(p0.z * wb.x + p0.w * wb.y + p1.w * f0b.y, p0.z * wb.y - p0.w * wb.x - p1.w * f0b.x);
            ch[2] = make_float2(p1.x * wb.x + p1.y * wb.y, p1.x * wb.y - p1.y * wb.x);
            ch[3] = make_float2(p2.y * bb.x + p2.x * f0b.x, p2.y * bb.y + p2.x * f0b.y);
        }
        for (int t = 0; t < nt; ++t) {
            const float2 v = ch[d.tq[t]];
            vt[t] = mk<T>(T(v.x), T(v.y));
        }
        return;
    }
    double s, c;
    sincos(d.omega[idx] * elapsed, &s, &c);
    const zd fpb = zload(Fpb + 2 * idx), fmb = zload(Fmb + 2 * idx), a0b = zload(F0b + 2 * idx);
    // cp_bar = Fp_bar * p ; cm_bar = Fm_bar * conj(p)
    const zd cpb{fpb.re * c - fpb.im * s, fpb.re * s + fpb.im * c};
    const zd cmb{fmb.re * c + fmb.im * s, fmb.im * c - fmb.re * s};
    const double k = d.k[w], l = d.l[w];
    const double vort = d.A0FromVorticity[idx], buoyF = d.A0FromBuoyancy[idx], na0 = d.NA0[idx], apmn = d.ApmN[idx];
    const zd waveb{cpb.re + cmb.re, cpb.im + cmb.im};
    const zd buoyb{cpb.re - cmb.re, cpb.im - cmb.im};
    const zd bvb{buoyb.re * apmn, buoyb.im * apmn};
    const zd a0cb{a0b.re - na0 * bvb.re, a0b.im - na0 * bvb.im};
    for (int t = 0; t < nt; ++t) {
        const int q = d.tq[t];
        double vr = 0.0, vi = 0.0;
        if (w == 0) {
            // inertial override: cp = f(value), cm = conj(cp)
            const double sc = d.inertialScale[j];
            const zd tot{cpb.re + cmb.re, cpb.im - cmb.im};  // cp_bar + conj(cm_bar)
            if (q == 0) { vr = sc * tot.re; vi = sc * tot.im; }
            if (q == 1) { vr = -sc * tot.im; vi = sc * tot.re; }  // (i sc) * tot
            if (q == 3) { vr += buoyF * a0b.re; vi += buoyF * a0b.im; }
        } else {
            if (q == 3) { vr += bvb.re; vi += bvb.im; }
            if (q == 0) { vr += -l * vort * a0cb.im; vi += l * vort * a0cb.re; }   // (i l) vort a0c_bar
            if (q == 1) { vr += k * vort * a0cb.im; vi += -k * vort * a0cb.re; }   // (-i k) vort a0c_bar
            if (q == 3) { vr += buoyF * a0cb.re; vi += buoyF * a0cb.im; }
            if (d.hydrostatic) {
                const zd apmd = zload(d.ApmD + 2 * idx);
                // conj(i kk ApmD) * wave_bar, kk = k (u) or l (v)
                const double kk = q == 0 ? k : (q == 1 ? l : 0.0);
                const zd cf{-kk * apmd.im, -kk * apmd.re};  // conj(i kk apmd) = -i kk conj(apmd)
                vr += cf.re * waveb.re - cf.im * waveb.im;
                vi += cf.re * waveb.im + cf.im * waveb.re;
            } else {
                if (q == 0) { const double sc = d.cosAlpha[w] * d.ApmDScaled[idx]; vr += sc * waveb.re; vi += sc * waveb.im; }
                if (q == 1) { const double sc = d.sinAlpha[w] * d.ApmDScaled[idx]; vr += sc * waveb.re; vi += sc * waveb.im; }
                if (q == 2) { const double sc = (d.Kh[w] / 2.0) * d.apmWPrefactor[j]; vr += sc * waveb.im; vi += -sc * waveb.re; }
            }
        }
        vt[t] = mk<T>(T(vr), T(vi));
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_vfwd_adj(DescDev d, const double* __restrict__ Fpb, const double* __restrict__ Fmb,
                                                 const double* __restrict__ F0b, double elapsed, cx<T>* __restrict__ zadj) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, nt = d.nt;
    const int m0 = blockIdx.x * kVfwdModes;
    const int nm = min(kVfwdModes, d.Nkl - m0);
    cx<T>* vb = reinterpret_cast<cx<T>*>(smem_raw);  // [nt][Nj][modes]
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mm = it % nm, j = it / nm;
        cx<T> vt[4];
        vfwd_adj_values<T>(d, Fpb, Fmb, F0b, elapsed, d.modeWV[m0 + mm], j, vt);
        for (int t = 0; t < nt; ++t) vb[(t * Nj + j) * kVfwdModes + mm] = vt[t];
    }
    __syncthreads();
    const T* Fc = reinterpret_cast<const T*>(d.FcosT);   // [Zh][Nj]
    const T* Fs = reinterpret_cast<const T*>(d.FsinT);
    for (int it = threadIdx.x; it < nm * Zh; it += blockDim.x) {
        const int n = it / nm, mm = it - n * nm;
        const int mode = m0 + mm;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const bool conj = d.modeFlags[mode] & 1;
        const int n2 = Nz - 1 - n;
        for (int t = 0; t < nt; ++t) {
            const bool cosine = d.tq[t] < 2;
            const T* F = cosine ? Fc : Fs;
            T E[2] = {T(0), T(0)}, O[2] = {T(0), T(0)};
            const T* Fn = F + (size_t)n * Nj;
            for (int j = 0; j < Nj; ++j) {
                const cx<T> v = vb[(t * Nj + j) * kVfwdModes + mm];
                const T f = Fn[j];
                if (j & 1) { O[0] += f * v.x; O[1] += f * v.y; } else { E[0] += f * v.x; E[1] += f * v.y; }
            }
            cx<T>* base = zadj + (size_t)t * Nz * P;
            cx<T> lo = mk<T>(E[0] + O[0], E[1] + O[1]);
            if (conj) lo.y = -lo.y;
            base[(size_t)n * P + pos] = lo;
            if (cpos >= 0) base[(size_t)n * P + cpos] = mk<T>(T(0), T(0));
            if (n2 != n) {
                cx<T> hi = cosine ? mk<T>(E[0] - O[0], E[1] - O[1]) : mk<T>(O[0] - E[0], O[1] - E[1]);
                if (conj) hi.y = -hi.y;
                base[(size_t)n2 * P + pos] = hi;
                if (cpos >= 0) base[(size_t)n2 * P + cpos] = mk<T>(T(0), T(0));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// x pass adjoint, one CTA per (y, z) row (shared-memory Stockham FFTs).

// physIn, when given, holds the forward real rows [z][nReal][y][Nx] (as
// k_xflux keeps them); otherwise they are recomputed from yspec.
//
// Like k_xflux, the row's forward spectra are read from L2 where the lines are
// built, and only what the product adjoint needs stays in shared memory: U, V,
// W and the adjoint rows S_q-bar (3 + nt rows); each derivative row is folded
// into the velocity gradients as soon as it is available, in row order
// (g_U -= S_q-bar q_x, g_V -= S_q-bar q_y, g_W -= S_q-bar q_z), and the
// derivative rows' own gradients (-S_q-bar U, -S_q-bar V, -S_q-bar W) are
// formed while their r2c lines are built.  About 69 KB of shared memory at
// Nx = 256 (paired FP32 / FP64), three CTAs per SM.
template <typename T>
__global__ void __launch_bounds__(256) k_xadj(DescDev d, const cx<T>* __restrict__ yspec, const cx<T>* __restrict__ yadj,
                                             cx<T>* __restrict__ yout, const T* __restrict__ physIn) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, KX = d.kxColumns, nt = d.nt, L = d.xLen;
    const int nIn = 4 + 2 * nt;
    const int nReal = 3 + 3 * nt;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);   // [L]
    cx<T>* twN = tw + L;                               // [Nx]
    cx<T>* specA = twN + Nx;                           // [nt][KX] adjoint spectra, interior kx halved
    cx<T>* out4 = specA + nt * KX;                     // [4][KX] output channels U, V, W, N
    cx<T>* bufA = out4 + 4 * KX;                       // [8][L]
    cx<T>* bufB = bufA + 8 * L;
    T* base = reinterpret_cast<T*>(bufB + 8 * L);     // [3 + nt][Nx]: U, V, W, then S_q-bar per target
    T* gacc = base + (3 + nt) * Nx;                    // [3][Nx]: gradients of U, V, W
    const cx<T>* yrow = yspec + ((size_t)z * nIn * Ny + y) * KX;
    const size_t cstride = (size_t)Ny * KX;
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) twN[i] = twgN[i];
    for (int i = threadIdx.x; i < nt * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        cx<T> v = yadj[(((size_t)z * nt + c) * Ny + y) * KX + k];
        if (k > 0) v = mk<T>(T(0.5) * v.x, T(0.5) * v.y);  // adjoint of r2c: interior kx at weight 1/2 under c2r
        specA[i] = v;
    }
    for (int i = threadIdx.x; i < 3 * Nx; i += blockDim.x) gacc[i] = T(0);
    if (physIn)
        for (int i = threadIdx.x; i < 3 * Nx; i += blockDim.x) {
            const int r = i / Nx, x = i - r * Nx;
            base[i] = physIn[(((size_t)z * nReal + r) * Ny + y) * Nx + x];
        }
    __syncthreads();
    auto rowSrc = [&](int r, int& ch, bool& useK) {
        if (r < 3) { ch = r; useK = false; return; }
        const int t = (r - 3) / 3, kind = (r - 3) % 3;
        const int q = d.tq[t];
        if (kind == 0) { ch = q; useK = true; }
        else if (kind == 1) { ch = 4 + t; useK = false; }
        else { ch = 4 + nt + t; useK = false; }
    };
    // c2r rows, in batches of 8: rows 0..2 U, V, W (unless kept), 3..2+nt the
    // adjoint rows S_q-bar, then the derivative rows q_x, q_y, q_z of each target
    // (unless kept), each folded into the gradients of U, V, W as it arrives
    auto rowOf = [&](int i) { return i < 3 ? i : (i < 3 + nt ? -1 - (i - 3) : i - nt); };  // -1 - t: adjoint row t
    const int nRows = nReal + nt;
    for (int rb = physIn ? 3 : 0; rb < nRows; rb += 8) {
        const int nr = physIn ? min(8, 3 + nt - rb) : min(8, nRows - rb);
        if (nr <= 0) break;
        for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
            const int li = i / L, k = i - li * L;
            const int r = rowOf(rb + li);
            if (r >= 0) {
                int ch; bool useK;
                rowSrc(r, ch, useK);
                bufA[li * L + k] = c2r_line_entry<T>(d, yrow + ch * cstride, k, useK, twN);
            } else {
                bufA[li * L + k] = c2r_line_entry<T>(d, specA + (-1 - r) * KX, k, false, twN);
            }
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, true>(bufA, bufB, d.fx, nr, L, tw);
        for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
            for (int li = 0; li < nr; ++li) {
                const int r = rowOf(rb + li);
                const T v = c2r_sample<T>(d, res + li * L, x);
                if (r < 0) base[(3 + (-1 - r)) * Nx + x] = v;
                else if (r < 3) base[r * Nx + x] = v;
                else {
                    const int t = (r - 3) / 3, kind = (r - 3) % 3;
                    gacc[kind * Nx + x] -= base[(3 + t) * Nx + x] * v;
                }
            }
        }
        __syncthreads();
    }
    if (physIn) {
        // kept derivative rows: folded in row order, as above
        for (int x = threadIdx.x; x < Nx; x += blockDim.x)
            for (int r = 3; r < nReal; ++r) {
                const int t = (r - 3) / 3, kind = (r - 3) % 3;
                const T v = physIn[(((size_t)z * nReal + r) * Ny + y) * Nx + x];
                gacc[kind * Nx + x] -= base[(3 + t) * Nx + x] * v;
            }
        __syncthreads();
    }
    // r2c of the gradient rows (adjoint of c2r: interior kx doubled): rows 0..2
    // the gradients of U, V, W, row 3 + 3 t + kind = -S_q-bar times U, V or W
    for (int rb = 0; rb < nReal; rb += 8) {
        const int nr = min(8, nReal - rb);
        for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
            const int li = i / L, n = i - li * L;
            const int r = rb + li;
            cx<T> e;
            if (r < 3) {
                e = r2c_line_entry<T>(d, gacc + r * Nx, n);
            } else {
                const int t = (r - 3) / 3, kind = (r - 3) % 3;
                const T* sb = base + (3 + t) * Nx;
                const T* vel = base + kind * Nx;
                if (d.xEven) e = mk<T>(-sb[2 * n] * vel[2 * n], -sb[2 * n + 1] * vel[2 * n + 1]);
                else e = mk<T>(-sb[n] * vel[n], T(0));
            }
            bufA[li * L + n] = e;
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, false>(bufA, bufB, d.fx, nr, L, tw);
        // one thread per kx walks the batch's rows in order: a channel's own row
        // (0..2) lands in out4 before its target's x-derivative row adds to it
        for (int k = threadIdx.x; k < KX; k += blockDim.x) {
            for (int li = 0; li < nr; ++li) {
                const int r = rb + li;
                cx<T> v = r2c_value<T>(d, res + li * L, k, twN);
                if (k > 0) v = mk<T>(T(2) * v.x, T(2) * v.y);
                // combine into the forward y-spectrum channel layout
                if (r < 3) {
                    out4[r * KX + k] = v;
                } else {
                    const int t = (r - 3) / 3, kind = (r - 3) % 3;
                    if (kind == 0) {  // x-derivative row of target q: (i k)^* = -i k onto channel q
                        const int c = d.tq[t];
                        const cx<T> base4 = c < 3 ? out4[c * KX + k] : mk<T>(T(0), T(0));
                        const T kk = row_k<T>(d)[k];
                        out4[c * KX + k] = mk<T>(base4.x + kk * v.y, base4.y - kk * v.x);
                    } else {
                        const int c = kind == 1 ? 4 + t : 4 + nt + t;
                        yout[(((size_t)z * nIn + c) * Ny + y) * KX + k] = v;
                    }
                }
            }
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < 4 * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        // channels without an x-derivative row (eta in the hydrostatic targets) get their own row or zero
        bool hasTarget = false;
        for (int t = 0; t < nt; ++t) hasTarget |= d.tq[t] == c;
        const cx<T> v = hasTarget || c < 3 ? out4[i] : mk<T>(T(0), T(0));
        yout[(((size_t)z * nIn + c) * Ny + y) * KX + k] = v;
    }
}

// ---------------------------------------------------------------------------
// y forward of the x-pass adjoint's output with the y-derivative channels folded
// back onto their source channel: out channel c = FFT_y(A) + (-i l) FFT_y(B)
// (B = -1: FFT_y(A) alone), gathered to the active rows -> fspec[c][z][pos].

template <typename T>
__global__ void __launch_bounds__(256) k_yfwd_pair(DescDev d, YFwdPairMap map, const cx<T>* __restrict__ pspec, int nIn,
                                                  cx<T>* __restrict__ fspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Ny = d.Ny, P = d.positions, KX = d.kxColumns;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* bufA = tw + Ny;
    cx<T>* bufB = bufA + kYG * Ny;
    cx<T>* keep = bufB + kYG * Ny;  // FFT of channel A while B is transformed
    const int kx0 = blockIdx.x * kYG;
    const int z = blockIdx.y;
    const int c = blockIdx.z;
    const int g = min(kYG, KX - kx0);
    const int a = map.srcA[c], b = map.srcB[c];
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twy);
    for (int i = threadIdx.x; i < Ny; i += blockDim.x) tw[i] = twg[i];
    auto load = [&](int ch) {
        const cx<T>* in = pspec + (((size_t)z * nIn + ch) * Ny) * KX;
        for (int i = threadIdx.x; i < g * Ny; i += blockDim.x) {
            const int y = i / g, gi = i - y * g;
            bufA[gi * Ny + y] = in[(size_t)y * KX + kx0 + gi];
        }
        __syncthreads();
    };
    load(a);
    cx<T>* res = fft_lines<T, false>(bufA, bufB, d.fy, g, Ny, tw);
    for (int i = threadIdx.x; i < g * Ny; i += blockDim.x) keep[i] = res[i];
    __syncthreads();
    cx<T>* resB = nullptr;
    if (b >= 0) {
        load(b);
        resB = fft_lines<T, false>(bufA, bufB, d.fy, g, Ny, tw);
    }
    cx<T>* out = fspec + ((size_t)c * d.zTotal + z) * P;
    const T* rl = row_l<T>(d);
    const int pBeg = d.colStart[kx0], pEnd = d.colStart[kx0 + g];
    for (int p = pBeg + threadIdx.x; p < pEnd; p += blockDim.x) {
        int gi = 0;
        while (gi + 1 < g && p >= d.colStart[kx0 + gi + 1]) ++gi;
        const int ky = d.posKy[p];
        cx<T> v = keep[gi * Ny + ky];
        if (b >= 0) {
            const cx<T> w = resB[gi * Ny + ky];
            const T l = rl[ky];
            v = mk<T>(v.x + l * w.y, v.y - l * w.x);
        }
        out[p] = v;
    }
}

// x r2c of field rows with interior kx doubled (adjoint of the inverse transform's c2r)
template <typename T>
__global__ void __launch_bounds__(256) k_xr2c_adj(DescDev d, const double* __restrict__ fields, int nch, cx<T>* __restrict__ pspec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, Nz = d.Nz, KX = d.kxColumns, L = d.xLen;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* twN = tw + L;
    cx<T>* bufA = twN + Nx;
    cx<T>* bufB = bufA + 4 * L;
    T* row = reinterpret_cast<T*>(bufB + 4 * L);
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
        cx<T> v = r2c_value<T>(d, res + t * L, k, twN);
        if (k > 0) v = mk<T>(T(2) * v.x, T(2) * v.y);
        pspec[(((size_t)z * nch + t) * Ny + y) * KX + k] = v;
    }
}

// ---------------------------------------------------------------------------
// vertical inverse adjoint + assembly adjoint.  FLUX: channels of the forward
// y-spectrum layout (U V W N, y-derivative per target, z-derivative per
// target); otherwise U V W N only (inverse transform).

// Retained columns per CTA of the transposed vertical inverse: 4 keeps its folded
// columns (8 channels x Zh x modes x 16 bytes in FP32) small enough for six CTAs
// per SM, which its latency-bound gathers need.
constexpr int kVinvAdjModes = 4;

// Assembly and phase of k_vinv transposed for one (mode, j): the field
// cotangents (ubT, vbT, wbT, nbT) -> (Ap, Am, A0) cotangents at index idx.
template <typename T>
__device__ __forceinline__ void vinv_adj_store(const DescDev& d, int idx, double elapsed, cx<T> ubT, cx<T> vbT, cx<T> wbT,
                                               cx<T> nbT, double* __restrict__ Apb, double* __restrict__ Amb,
                                               double* __restrict__ A0b) {
    if constexpr (sizeof(T) == 4) {
        // MIXED: assembly adjoint with the FP32 field factors, FP32 phase after
        // FP64 angle reduction
        const float2 uap = *reinterpret_cast<const float2*>(d.fUAp + 2 * idx);
        const float2 vap = *reinterpret_cast<const float2*>(d.fVAp + 2 * idx);
        const float2 wap = *reinterpret_cast<const float2*>(d.fWAp + 2 * idx);
        const float2 ua0 = *reinterpret_cast<const float2*>(d.fUA0 + 2 * idx);
        const float2 va0 = *reinterpret_cast<const float2*>(d.fVA0 + 2 * idx);
        const float nap = d.fNAp[idx], na0 = d.fNA0[idx];
        auto cm = [](float2 a, cx<T> b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto cjm = [](float2 a, cx<T> b) { return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); };
        const float2 t1 = cjm(uap, ubT), t2 = cjm(vap, vbT), t3 = cjm(wap, wbT);
        const float2 ape = make_float2(t1.x + t2.x + t3.x + nap * nbT.x, t1.y + t2.y + t3.y + nap * nbT.y);
        const float2 s1 = cm(uap, ubT), s2 = cm(vap, vbT);
        const float2 ame = make_float2(s1.x + s2.x + t3.x - nap * nbT.x, s1.y + s2.y + t3.y - nap * nbT.y);
        const float2 r1 = cjm(ua0, ubT), r2 = cjm(va0, vbT);
        const float2 a0 = make_float2(r1.x + r2.x + na0 * nbT.x, r1.y + r2.y + na0 * nbT.y);
        const double ang = d.omega[idx] * elapsed;
        const double red = ang - 6.283185307179586476925 * rint(ang * 0.15915494309189533577);
        float sn, cs;
        sincosf(float(red), &sn, &cs);
        Apb[2 * idx] = double(ape.x * cs + ape.y * sn);   // ape * conj(p)
        Apb[2 * idx + 1] = double(ape.y * cs - ape.x * sn);
        Amb[2 * idx] = double(ame.x * cs - ame.y * sn);   // ame * p
        Amb[2 * idx + 1] = double(ame.x * sn + ame.y * cs);
        A0b[2 * idx] = double(a0.x);
        A0b[2 * idx + 1] = double(a0.y);
        return;
    }
    const zd ub{double(ubT.x), double(ubT.y)}, vbv{double(vbT.x), double(vbT.y)};
    const zd wb{double(wbT.x), double(wbT.y)}, nb{double(nbT.x), double(nbT.y)};
    // assembly adjoint (coefficientValueForField on evolved coefficients)
    const zd uap = zload(d.UAp + 2 * idx), vap = zload(d.VAp + 2 * idx), wap = zload(d.WAp + 2 * idx);
    const zd ua0 = zload(d.UA0 + 2 * idx), va0 = zload(d.VA0 + 2 * idx);
    const double nap = d.NAp[idx], na0 = d.NA0[idx];
    const zd ape = zadd(zadd(zadd(zmul(zconj(uap), ub), zmul(zconj(vap), vbv)), zmul(zconj(wap), wb)), zscale(nb, nap));
    const zd ame = zsub(zadd(zadd(zmul(uap, ub), zmul(vap, vbv)), zmul(zconj(wap), wb)), zscale(nb, nap));
    const zd a0 = zadd(zadd(zmul(zconj(ua0), ub), zmul(zconj(va0), vbv)), zscale(nb, na0));
    double s, c;
    sincos(d.omega[idx] * elapsed, &s, &c);
    zstore(Apb + 2 * idx, zmul(ape, zd{c, -s}));
    zstore(Amb + 2 * idx, zmul(ame, zd{c, s}));
    zstore(A0b + 2 * idx, a0);
}

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256) k_vinv_adj(DescDev d, const cx<T>* __restrict__ fadj, int nchIn, double elapsed,
                                                 double* __restrict__ Apb, double* __restrict__ Amb, double* __restrict__ A0b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, nt = d.nt;
    const int m0 = blockIdx.x * kVinvAdjModes;
    const int nm = min(kVinvAdjModes, d.Nkl - m0);
    const int nOutCh = FLUX ? 4 + nt : 4;  // value channels U V W N, then z-derivative per target
    cx2t<T>* pq = reinterpret_cast<cx2t<T>*>(smem_raw);  // [nOutCh][Zh][modes]
    // gather (stored rows + conjugated completion rows, -i l on y-derivative channels), fold z <-> Nz-1-z
    for (int it = threadIdx.x; it < nOutCh * Zh * nm; it += blockDim.x) {
        const int mm = it % nm;
        const int rest = it / nm;
        const int n = rest % Zh, oc = rest / Zh;
        const int mode = m0 + mm;
        const int pos = d.modePos[mode], cpos = d.modeCompPos[mode];
        const unsigned char flags = d.modeFlags[mode];
        // FLUX input is folded by k_yfwd_pair: value channels 0..3 already carry their
        // (-i l) y-derivative parts, z-derivative channels follow at 4..4+nt
        const int ch = oc;
        auto rowval = [&](int p, int zz) -> cx<T> { return fadj[((size_t)ch * Nz + zz) * P + p]; };
        auto colval = [&](int zz) -> cx<T> {
            cx<T> v = rowval(pos, zz);
            if (cpos >= 0) { const cx<T> c = rowval(cpos, zz); v = mk<T>(v.x + c.x, v.y - c.y); }
            if (flags & 2) v.y = T(0);
            if (flags & 1) v.y = -v.y;
            return v;
        };
        const cx<T> a = colval(n);
        const int n2 = Nz - 1 - n;
        cx2t<T> v;
        if (n2 == n) { v.p = a; v.q = a; }
        else { const cx<T> b = colval(n2); v.p = cadd<T>(a, b); v.q = csub<T>(a, b); }
        pq[(oc * Zh + n) * kVinvAdjModes + mm] = v;
    }
    __syncthreads();
    const T* Cc = reinterpret_cast<const T*>(d.CcosT);   // [Nj][Zh]
    const T* Cs = reinterpret_cast<const T*>(d.CsinT);
    const T* Ccm = reinterpret_cast<const T*>(d.CcosMT);
    const T* Csm = reinterpret_cast<const T*>(d.CsinMT);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mm = it % nm, j = it / nm;
        const int w = d.modeWV[m0 + mm];
        const int idx = j + Nj * w;
        const bool evenJ = (j & 1) == 0;
        // transposed inverse matrices: cos family uses (S_n + S_{N-1-n}) for even j
        auto contract = [&](int oc, const T* C, bool cosine) -> cx<T> {
            const bool useP = cosine ? evenJ : !evenJ;
            T re = T(0), im = T(0);
            const cx2t<T>* col = pq + (size_t)oc * Zh * kVinvAdjModes + mm;
            const T* Cj = C + (size_t)j * Zh;
            for (int n = 0; n < Zh; ++n) {
                const cx2t<T> v = col[n * kVinvAdjModes];
                const T f = Cj[n];
                const cx<T> sv = useP ? v.p : v.q;
                re += f * sv.x;
                im += f * sv.y;
            }
            return mk<T>(re, im);
        };
        cx<T> ubT = contract(0, Cc, true), vbT = contract(1, Cc, true), wbT = contract(2, Cs, false), nbT = contract(3, Cs, false);
        if (FLUX) {
            for (int t = 0; t < nt; ++t) {
                const int q = d.tq[t];
                const cx<T> zb = (q < 2) ? contract(4 + t, Csm, false) : contract(4 + t, Ccm, true);
                if (q == 0) ubT = cadd<T>(ubT, zb);
                if (q == 1) vbT = cadd<T>(vbT, zb);
                if (q == 2) wbT = cadd<T>(wbT, zb);
                if (q == 3) nbT = cadd<T>(nbT, zb);
            }
        }
        vinv_adj_store<T>(d, idx, elapsed, ubT, vbT, wbT, nbT, Apb, Amb, A0b);
    }
}

}  // namespace dev
}  // namespace wvgpu

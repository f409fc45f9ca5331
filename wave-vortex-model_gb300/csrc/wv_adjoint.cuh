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
        const int w = d.modeWV[m0 + mm];
        const int idx = j + Nj * w;
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
            vb[(t * Nj + j) * kVfwdModes + mm] = mk<T>(T(vr), T(vi));
        }
    }
    __syncthreads();
    const T* Fc = reinterpret_cast<const T*>(d.Fcos);
    const T* Fs = reinterpret_cast<const T*>(d.Fsin);
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
            for (int j = 0; j < Nj; ++j) {
                const cx<T> v = vb[(t * Nj + j) * kVfwdModes + mm];
                const T f = F[(size_t)j * Zh + n];
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

template <typename T>
__global__ void __launch_bounds__(256) k_xadj(DescDev d, const cx<T>* __restrict__ yspec, const cx<T>* __restrict__ yadj,
                                             cx<T>* __restrict__ yout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nx = d.Nx, Ny = d.Ny, KX = d.kxColumns, nt = d.nt, L = d.xLen;
    const int nIn = 4 + 2 * nt;
    const int nReal = 3 + 3 * nt;
    const int y = blockIdx.x, z = blockIdx.y;
    cx<T>* tw = reinterpret_cast<cx<T>*>(smem_raw);   // [L]
    cx<T>* twN = tw + L;                               // [Nx]
    cx<T>* specF = twN + Nx;                           // [nIn][KX]
    cx<T>* specA = specF + nIn * KX;                   // [nt][KX]
    cx<T>* bufA = specA + nt * KX;                     // [8][L]
    cx<T>* bufB = bufA + 8 * L;
    T* phys = reinterpret_cast<T*>(bufB + 8 * L);     // [nReal][Nx] forward rows
    T* sbar = phys + nReal * Nx;                       // [nt][Nx]
    T* grad = sbar + nt * Nx;                          // [nReal][Nx]
    const cx<T>* twg = reinterpret_cast<const cx<T>*>(d.twx);
    const cx<T>* twgN = reinterpret_cast<const cx<T>*>(d.twxN);
    for (int i = threadIdx.x; i < L; i += blockDim.x) tw[i] = twg[i];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) twN[i] = twgN[i];
    for (int i = threadIdx.x; i < nIn * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        specF[i] = yspec[(((size_t)z * nIn + c) * Ny + y) * KX + k];
    }
    for (int i = threadIdx.x; i < nt * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        cx<T> v = yadj[(((size_t)z * nt + c) * Ny + y) * KX + k];
        if (k > 0) v = mk<T>(T(0.5) * v.x, T(0.5) * v.y);  // adjoint of r2c: interior kx at weight 1/2 under c2r
        specA[i] = v;
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
    // c2r: forward rows (nReal) then adjoint rows (nt)
    const int nC2R = nReal + nt;
    for (int rb = 0; rb < nC2R; rb += 8) {
        const int nr = min(8, nC2R - rb);
        for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
            const int li = i / L, k = i - li * L;
            const int r = rb + li;
            if (r < nReal) {
                int ch; bool useK;
                rowSrc(r, ch, useK);
                bufA[li * L + k] = c2r_line_entry<T>(d, specF + ch * KX, k, useK, twN);
            } else {
                bufA[li * L + k] = c2r_line_entry<T>(d, specA + (r - nReal) * KX, k, false, twN);
            }
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, true>(bufA, bufB, d.fx, nr, L, tw);
        for (int i = threadIdx.x; i < nr * Nx; i += blockDim.x) {
            const int li = i / Nx, x = i - li * Nx;
            const int r = rb + li;
            const T v = c2r_sample<T>(d, res + li * L, x);
            if (r < nReal) phys[r * Nx + x] = v; else sbar[(r - nReal) * Nx + x] = v;
        }
        __syncthreads();
    }
    // product adjoint: S_q = -(U q_x + V q_y + W q_z)
    for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
        const T U = phys[0 * Nx + x], V = phys[1 * Nx + x], W = phys[2 * Nx + x];
        T gu = T(0), gv = T(0), gw = T(0);
        for (int t = 0; t < nt; ++t) {
            const T sb = sbar[t * Nx + x];
            gu -= sb * phys[(3 + 3 * t) * Nx + x];
            gv -= sb * phys[(4 + 3 * t) * Nx + x];
            gw -= sb * phys[(5 + 3 * t) * Nx + x];
            grad[(3 + 3 * t) * Nx + x] = -sb * U;
            grad[(4 + 3 * t) * Nx + x] = -sb * V;
            grad[(5 + 3 * t) * Nx + x] = -sb * W;
        }
        grad[0 * Nx + x] = gu;
        grad[1 * Nx + x] = gv;
        grad[2 * Nx + x] = gw;
    }
    __syncthreads();
    // r2c of the gradient rows (adjoint of c2r: interior kx doubled); results kept in specF (reused)
    cx<T>* gspec = specF;  // [nReal][KX] (nReal*KX <= nIn*KX + nt*KX: specF and specA are contiguous)
    for (int rb = 0; rb < nReal; rb += 8) {
        const int nr = min(8, nReal - rb);
        for (int i = threadIdx.x; i < nr * L; i += blockDim.x) {
            const int li = i / L, n = i - li * L;
            bufA[li * L + n] = r2c_line_entry<T>(d, grad + (rb + li) * Nx, n);
        }
        __syncthreads();
        cx<T>* res = fft_lines<T, false>(bufA, bufB, d.fx, nr, L, tw);
        for (int i = threadIdx.x; i < nr * KX; i += blockDim.x) {
            const int li = i / KX, k = i - li * KX;
            cx<T> v = r2c_value<T>(d, res + li * L, k, twN);
            if (k > 0) v = mk<T>(T(2) * v.x, T(2) * v.y);
            gspec[(rb + li) * KX + k] = v;
        }
        __syncthreads();
    }
    // combine into the forward y-spectrum channel layout
    for (int i = threadIdx.x; i < nIn * KX; i += blockDim.x) {
        const int c = i / KX, k = i - c * KX;
        cx<T> v = mk<T>(T(0), T(0));
        if (c < 4) {
            if (c < 3) v = gspec[c * KX + k];
            for (int t = 0; t < nt; ++t) {
                if (d.tq[t] == c) {  // x-derivative row of target c: (i k)^* = -i k
                    const cx<T> g = gspec[(3 + 3 * t) * KX + k];
                    const T kk = row_k<T>(d)[k];
                    v = mk<T>(v.x + kk * g.y, v.y - kk * g.x);
                }
            }
        } else if (c < 4 + nt) {
            v = gspec[(4 + 3 * (c - 4)) * KX + k];
        } else {
            v = gspec[(5 + 3 * (c - 4 - nt)) * KX + k];
        }
        yout[(((size_t)z * nIn + c) * Ny + y) * KX + k] = v;
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

template <typename T, bool FLUX>
__global__ void __launch_bounds__(256) k_vinv_adj(DescDev d, const cx<T>* __restrict__ fadj, int nchIn, double elapsed,
                                                 double* __restrict__ Apb, double* __restrict__ Amb, double* __restrict__ A0b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Nj = d.Nj, Nz = d.Nz, Zh = d.zHalf, P = d.positions, nt = d.nt;
    const int m0 = blockIdx.x * kVinvModes;
    const int nm = min(kVinvModes, d.Nkl - m0);
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
        int ch = oc, ych = -1;
        if (oc < 4) {
            if (FLUX)
                for (int t = 0; t < nt; ++t) if (d.tq[t] == oc) ych = 4 + t;
        } else {
            ch = 4 + nt + (oc - 4);
        }
        auto rowval = [&](int p, int zz) -> cx<T> {
            cx<T> v = fadj[((size_t)ch * Nz + zz) * P + p];
            if (ych >= 0) {
                const cx<T> g = fadj[((size_t)ych * Nz + zz) * P + p];
                const T l = row_l<T>(d)[d.posKy[p]];
                v = mk<T>(v.x + l * g.y, v.y - l * g.x);  // + (-i l) g
            }
            return v;
        };
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
        pq[(oc * Zh + n) * kVinvModes + mm] = v;
    }
    __syncthreads();
    const T* Cc = reinterpret_cast<const T*>(d.Ccos);
    const T* Cs = reinterpret_cast<const T*>(d.Csin);
    const T* Ccm = reinterpret_cast<const T*>(d.CcosM);
    const T* Csm = reinterpret_cast<const T*>(d.CsinM);
    for (int it = threadIdx.x; it < nm * Nj; it += blockDim.x) {
        const int mm = it % nm, j = it / nm;
        const int w = d.modeWV[m0 + mm];
        const int idx = j + Nj * w;
        const bool evenJ = (j & 1) == 0;
        // transposed inverse matrices: cos family uses (S_n + S_{N-1-n}) for even j
        auto contract = [&](int oc, const T* C, bool cosine) -> zd {
            const bool useP = cosine ? evenJ : !evenJ;
            T re = T(0), im = T(0);
            const cx2t<T>* col = pq + (size_t)oc * Zh * kVinvModes + mm;
            for (int n = 0; n < Zh; ++n) {
                const cx2t<T> v = col[n * kVinvModes];
                const T f = C[(size_t)n * Nj + j];
                const cx<T> sv = useP ? v.p : v.q;
                re += f * sv.x;
                im += f * sv.y;
            }
            return zd{double(re), double(im)};
        };
        zd ub = contract(0, Cc, true), vbv = contract(1, Cc, true), wb = contract(2, Cs, false), nb = contract(3, Cs, false);
        if (FLUX) {
            for (int t = 0; t < nt; ++t) {
                const int q = d.tq[t];
                const zd zb = (q < 2) ? contract(4 + t, Csm, false) : contract(4 + t, Ccm, true);
                if (q == 0) ub = zadd(ub, zb);
                if (q == 1) vbv = zadd(vbv, zb);
                if (q == 2) wb = zadd(wb, zb);
                if (q == 3) nb = zadd(nb, zb);
            }
        }
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
}

}  // namespace dev
}  // namespace wvgpu

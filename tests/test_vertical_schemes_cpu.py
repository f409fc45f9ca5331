"""CPU models of the arithmetic the vertical-transform kernels rely on, checked
against the oracle's matrices (no GPU):

* the even / odd extension FFTs of k_vinv_fft, k_vfwd_fft and their adjoints
  (k_vinv_adj_fft, k_vfwd_adj_fft): one complex FFT of 2(Nz-1) points carries
  a cosine-family and a sine-family channel, and the even / odd parts of the
  result reproduce Ccos / Csin, Fcos / Fsin and their transposes;
* the digit slicing of k_vinv_tcx: six balanced base-256 digits per row-scaled
  value (every digit in [-128, 128], reconstruction within 2^-48 of the row
  scale), level sums that stay exact in FP32, and the contraction accuracy with
  m_j taken on the A side of the z-derivative matrices."""
import numpy as np
import pytest

import wv_oracle as O


def _desc(Nz, Nj=None):
    c = O.Config(Nx=16, Ny=16, Nz=Nz, Nj=Nj or O.default_nj(Nz), Lx=50e3, Ly=50e3, Lz=4000.0, latitude=33.0)
    return c, O.build_descriptor(c)


def _even_odd(F, L, N2, n):
    if n in (0, L):
        return F[n], 0.0
    return (F[n] + F[N2 - n]) / 2, (F[n] - F[N2 - n]) / 2


@pytest.mark.parametrize("Nz", [7, 17, 24, 64, 129])
def test_fft_inverse_and_forward_match_the_matrices(Nz):
    c, d = _desc(Nz)
    ccos, csin, _, _ = O._inverse_matrices(d)   # (Nz, Nj)
    fc, fs = O._forward_matrices(d)             # (Nj, Nz)
    L, N2, Nj = Nz - 1, 2 * (Nz - 1), c.Nj
    rng = np.random.default_rng(Nz)
    C = rng.standard_normal(Nj) + 1j * rng.standard_normal(Nj)
    D = rng.standard_normal(Nj) + 1j * rng.standard_normal(Nj)
    # inverse (k_vinv_fft): y[0] = C0/2, y[j] = (C + iD)/2, y[2L-j] = (C - iD)/2
    y = np.zeros(N2, complex)
    y[0] = C[0] / 2
    for j in range(1, Nj):
        y[j] = (C[j] + 1j * D[j]) / 2
        y[N2 - j] = (C[j] - 1j * D[j]) / 2
    F = np.fft.fft(y)
    ev, od = zip(*(_even_odd(F, L, N2, n) for n in range(L + 1)))
    assert np.abs(np.array(ev) - ccos @ C).max() <= 1e-14 * np.abs(ccos @ C).max()
    assert np.abs(np.array(od) - csin @ D).max() <= 1e-14 * np.abs(csin @ D).max()
    # forward (k_vfwd_fft): y[0] = c0, y[L] = cL, y[z] = c + s, y[2L-z] = c - s; X = E / (L Nx Ny), i O / (L Nx Ny)
    cz = rng.standard_normal(Nz) + 1j * rng.standard_normal(Nz)
    sz = rng.standard_normal(Nz) + 1j * rng.standard_normal(Nz)
    y = np.zeros(N2, complex)
    y[0], y[L] = cz[0], cz[L]
    for z in range(1, L):
        y[z], y[N2 - z] = cz[z] + sz[z], cz[z] - sz[z]
    F = np.fft.fft(y)
    sc = 1.0 / (L * c.Nx * c.Ny)
    Xc = np.array([_even_odd(F, L, N2, j)[0] * sc for j in range(Nj)])
    Xs = np.array([1j * _even_odd(F, L, N2, j)[1] * sc for j in range(Nj)])
    assert np.abs(Xc - fc @ cz).max() <= 1e-14 * np.abs(fc @ cz).max()
    assert np.abs(Xs - fs @ sz).max() <= 1e-14 * np.abs(fs @ sz).max()


@pytest.mark.parametrize("Nz", [9, 24, 65])
def test_fft_adjoint_lines_are_the_transposes(Nz):
    c, d = _desc(Nz)
    ccos, csin, _, _ = O._inverse_matrices(d)
    fc, fs = O._forward_matrices(d)
    L, N2, Nj = Nz - 1, 2 * (Nz - 1), c.Nj
    rng = np.random.default_rng(100 + Nz)
    # k_vfwd_adj_fft: inverse-type line, cosine part scaled by w_z / (L Nx Ny), sine part by 2 / (L Nx Ny)
    Xc = rng.standard_normal(Nj) + 1j * rng.standard_normal(Nj)
    Xs = rng.standard_normal(Nj) + 1j * rng.standard_normal(Nj)
    y = np.zeros(N2, complex)
    y[0] = Xc[0]
    for j in range(1, Nj):
        y[j] = (Xc[j] + 1j * Xs[j]) / 2
        y[N2 - j] = (Xc[j] - 1j * Xs[j]) / 2
    F = np.fft.fft(y)
    sc = 1.0 / (L * c.Nx * c.Ny)
    xc = np.array([(F[z] * sc) if z in (0, L) else (F[z] + F[N2 - z]) * sc for z in range(Nz)])
    xs = np.array([0.0 if z in (0, L) else (F[z] - F[N2 - z]) / 2 * 2 * sc for z in range(Nz)])
    assert np.abs(xc - fc.T @ Xc).max() <= 1e-14 * np.abs(fc.T @ Xc).max()
    assert np.abs(xs - fs.T @ Xs).max() <= 1e-14 * np.abs(fs.T @ Xs).max()
    # k_vinv_adj_fft: forward-type line y[0] = o0, y[L] = oL, y[z] = (o + i s)/2; Ccos's 1/2 at j = 0
    o = rng.standard_normal(Nz) + 1j * rng.standard_normal(Nz)
    s = rng.standard_normal(Nz) + 1j * rng.standard_normal(Nz)
    y = np.zeros(N2, complex)
    y[0], y[L] = o[0], o[L]
    for z in range(1, L):
        y[z], y[N2 - z] = (o[z] + 1j * s[z]) / 2, (o[z] - 1j * s[z]) / 2
    F = np.fft.fft(y)
    Cb = np.array([_even_odd(F, L, N2, j)[0] * (0.5 if j == 0 else 1.0) for j in range(Nj)])
    Db = np.array([_even_odd(F, L, N2, j)[1] for j in range(Nj)])
    assert np.abs(Cb - ccos.T @ o).max() <= 1e-14 * np.abs(ccos.T @ o).max()
    assert np.abs(Db - csin.T @ s).max() <= 1e-14 * np.abs(csin.T @ s).max()


def _digits(Y, S=6):
    """Balanced base-256 digits of integers |Y| <= 2^47, least significant last."""
    D = np.zeros((S,) + Y.shape, dtype=np.int64)
    Y = Y.copy()
    for s in range(S - 1, 0, -1):
        dd = Y & 0xFF
        dd = dd - ((dd & 0x80) << 1)
        D[s] = dd
        Y = (Y - dd) // 256
    D[0] = Y
    return D


def _split_rows(X):
    mx = np.abs(X).max(axis=1)
    E = np.where(mx > 0, np.frexp(mx)[1], 0)
    Y = np.rint(np.ldexp(X, (47 - E)[:, None])).astype(np.int64)
    D = _digits(Y)
    slices = np.array([np.ldexp(D[s].astype(np.float64), -7 - 8 * s) for s in range(6)])
    return D, slices, E


def test_digit_slices_are_exact_and_bounded():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((64, 85)) * 10.0 ** rng.integers(-8, 8, size=(64, 1))
    D, slices, E = _split_rows(X)
    assert np.abs(D).max() <= 128
    rec = np.ldexp(slices.sum(axis=0), E[:, None])
    scale = np.ldexp(1.0, E)[:, None]
    assert np.max(np.abs(rec - X) / scale) <= 2.0 ** -48
    # every slice value is exact in BF16 (at most 8 significant bits)
    for s in range(6):
        m, _ = np.frexp(slices[s])
        assert np.all(np.abs(np.ldexp(m, 8) - np.rint(np.ldexp(m, 8))) == 0)


def _contract(S, Cm, levels_exact=3):
    """The k_vinv_tcx contraction of rows S (over j) with rows Cm (over j) per
    parity of j: accumulators of levels 0 .. levels_exact-1 and one for the
    rest, each summed in FP32; returns the result and whether the exact levels
    stayed exact."""
    a, E = _split_rows(S)[1:]
    b, F = _split_rows(Cm)[1:]
    Nj = S.shape[1]
    out = np.zeros((S.shape[0], Cm.shape[0]), complex if np.iscomplexobj(S) else float)
    exact = True
    for par in (0, 1):
        js = np.arange(par, Nj, 2)
        acc = [np.zeros(out.shape, np.float32) for _ in range(levels_exact + 1)]
        ref = [np.zeros(out.shape) for _ in range(levels_exact + 1)]
        for lv in range(5, -1, -1):
            for s in range(lv + 1):
                t = lv - s
                P = a[s][:, js][:, None, :] * b[t][:, js][None, :, :]
                k = min(lv, levels_exact)
                for q in range(P.shape[2]):
                    acc[k] = (acc[k] + P[:, :, q].astype(np.float32)).astype(np.float32)
                    ref[k] = ref[k] + P[:, :, q]
        for k in range(levels_exact):
            exact &= bool(np.array_equal(acc[k].astype(np.float64), ref[k]))
        out += np.ldexp(sum(x.astype(np.float64) for x in acc), E[:, None] + F[None, :])
    return out, exact


def test_digit_sliced_contraction_accuracy():
    c, d = _desc(129)
    ccos, csin, _, _ = O._inverse_matrices(d)
    Zh = (c.Nz + 1) // 2
    m = d.m[:c.Nj]
    rng = np.random.default_rng(1)
    S = rng.standard_normal((32, c.Nj)) * (np.arange(c.Nj) + 1.0) ** -1.5 * 1e-2
    for C, A in ((ccos[:Zh], S), (csin[:Zh], S), (ccos[:Zh], S * m), (-csin[:Zh], S * m)):
        exact = A @ C.T
        got, levels_exact = _contract(A, C)
        assert levels_exact
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) <= 1e-12
    # with m_j on the matrix side instead the error bound (relative to
    # max|a| max|b|) loses two orders of magnitude: the reason for the A side
    Cm = -m[None, :] * csin[:Zh]
    exact = S @ Cm.T
    got, _ = _contract(S, Cm, levels_exact=2)
    assert np.linalg.norm(got - exact) / np.linalg.norm(exact) > 1e-11

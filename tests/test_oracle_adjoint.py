"""The oracle's hand-written adjoint (flux, inverse transform, RK4 step):
dot-product tests against central differences, which are exact for the
quadratic flux up to rounding.  The GPU adjoint is checked against it."""
import numpy as np
import pytest

import wv_oracle as O

ADJ_CASES = [
    O.Config(Nx=16, Ny=16, Nz=9, Nj=5, Lx=40e3, Ly=40e3, Lz=1000.0, latitude=45.0),
    O.Config(Nx=15, Ny=13, Nz=9, Nj=5, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0),
    O.Config(Nx=8, Ny=6, Nz=7, Nj=4, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0, isHydrostatic=True),
]


def cplx(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def inner(a, b):
    return sum(float(np.real(np.vdot(x, y))) for x, y in zip(a, b))


@pytest.mark.parametrize("c", ADJ_CASES, ids=lambda c: f"{c.Nx}x{c.Ny}x{c.Nz}{'h' if c.isHydrostatic else ''}")
def test_flux_and_inverse_dot_product(c):
    rng = np.random.default_rng(1)
    d = O.build_descriptor(c)
    sh = (d.Nkl, c.Nj)
    A = [1e-3 * cplx(rng, sh) for _ in range(3)]
    dA = [cplx(rng, sh) for _ in range(3)]
    Fb = [cplx(rng, sh) for _ in range(3)]
    t, t0, eps = 123.0, 7.0, 1e-3
    Fp = O.nonlinear_flux(d, *[A[i] + eps * dA[i] for i in range(3)], t, t0)
    Fm = O.nonlinear_flux(d, *[A[i] - eps * dA[i] for i in range(3)], t, t0)
    jvp = [(Fp[i] - Fm[i]) / (2 * eps) for i in range(3)]
    lhs = inner(Fb, jvp)
    rhs = inner(O.flux_vjp(d, *A, t, t0, *Fb), dA)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    fb = rng.standard_normal((4, c.Nz, c.Ny, c.Nx))
    l2 = float(np.sum(fb * O.inverse_uvweta(d, *dA, t, t0)))
    r2 = inner(O.inverse_vjp(d, t, t0, fb), dA)
    assert abs(l2 - r2) <= 1e-12 * abs(l2)


def test_rk4_step_adjoint_matches_central_differences():
    c = ADJ_CASES[0]
    rng = np.random.default_rng(2)
    d = O.build_descriptor(c)
    sh = (d.Nkl, c.Nj)
    A = [1e-2 * cplx(rng, sh) for _ in range(3)]
    dA = [cplx(rng, sh) for _ in range(3)]
    yb = [cplx(rng, sh) for _ in range(3)]
    h = 30.0

    def central(eps):
        Yp = O.rk4_step(d, *[A[i] + eps * dA[i] for i in range(3)], 0.0, 0.0, h)
        Ym = O.rk4_step(d, *[A[i] - eps * dA[i] for i in range(3)], 0.0, 0.0, h)
        return inner(yb, [(Yp[i] - Ym[i]) / (2 * eps) for i in range(3)])

    # the RK4 map is a polynomial of degree 16: Richardson-extrapolate the O(eps^2) term
    fd = (4.0 * central(5e-6) - central(1e-5)) / 3.0
    adj = inner(O.rk4_step_vjp(d, *A, 0.0, 0.0, h, yb), dA)
    assert abs(fd - adj) <= 1e-8 * abs(adj)

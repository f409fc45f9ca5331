"""GPU adjoint (vector-Jacobian products) through the C ABI.  No reference
counterpart: checked against the oracle's adjoint (itself checked by
dot-product tests), by GPU dot-product tests (central differences are exact for
the quadratic flux up to rounding), and by finite differences of a misfit
J = 0.5 ||(u, v, eta)(T) - target||^2 through RK4."""
import numpy as np
import pytest

import wv_oracle as O
from _cases import FP64_REL_TOL, config_from_case, golden_cases, load_golden, parity_tolerance, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available()
    build.build()
    return wvgpu


def to_wv(wv, c):
    return wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                            planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                            isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.cpu().numpy()


def inner(a, b):
    return sum(float(np.real(np.vdot(x, y))) for x, y in zip(a, b))


def cplx(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("name", ["wave_16x16x9", "odd_15x13x9", "hydro_8x6x7", "noalias_16x16x9"])
def test_flux_vjp_matches_oracle_adjoint(wv, name):
    cf = golden_cases()[name]
    c = config_from_case(cf)
    d = O.build_descriptor(c)
    g = load_golden(name)
    rng = np.random.default_rng(3)
    Fb = [cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    t, t0 = float(g["t"]), float(g["t0"])
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    got = k.flux_vjp(t, t0, *(dev(g[n]) for n in ("Ap", "Am", "A0")), *(dev(x) for x in Fb))
    ref = O.flux_vjp(d, g["Ap"], g["Am"], g["A0"], t, t0, *Fb)
    for a, b in zip(got, ref):
        assert rel_err(host(a), b) <= FP64_REL_TOL
    k.close()


@pytest.mark.parametrize("shape,hydro", [((64, 64, 33), False), ((48, 40, 17), True)])
def test_flux_vjp_dot_product_on_gpu(wv, shape, hydro):
    """<Fbar, dF> = <VJP(Fbar), dA> with dF from central differences of the GPU flux
    (exact for the quadratic flux up to rounding)."""
    Nx, Ny, Nz = shape
    c = O.Config(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=400e3, Ly=400e3 * Ny / Nx, Lz=4000.0, latitude=33.0,
                 isHydrostatic=hydro)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(4)
    A = O.spectrum_state(d, seed=9, urms=0.1)
    scale = max(float(np.max(np.abs(x))) for x in A)
    dA = [scale * cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    Fb = [cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    t, t0, eps = 500.0, 0.0, 1e-2
    Fp = k.nonlinearFlux(t, t0, *[A[i] + eps * dA[i] for i in range(3)])
    Fm = k.nonlinearFlux(t, t0, *[A[i] - eps * dA[i] for i in range(3)])
    lhs = inner(Fb, [(Fp[i] - Fm[i]) / (2 * eps) for i in range(3)])
    vjp = k.flux_vjp(t, t0, *(dev(x) for x in A), *(dev(x) for x in Fb))
    rhs = inner([host(x) for x in vjp], dA)
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)
    # and against the oracle's adjoint within its FP64 noise floor
    ref, floors = O.noise_floor(O.flux_vjp, d, *A, t, t0, *Fb)
    for a, b, fl in zip(vjp, ref, floors):
        assert rel_err(host(a), b) <= parity_tolerance(fl), (rel_err(host(a), b), fl)
    k.close()


@pytest.mark.parametrize("name", ["wave_16x16x9", "odd_15x13x9"])
def test_inverse_vjp_matches_oracle(wv, name):
    import torch
    c = config_from_case(golden_cases()[name])
    d = O.build_descriptor(c)
    rng = np.random.default_rng(5)
    fb = rng.standard_normal((4, c.Nz, c.Ny, c.Nx))
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    got = k.inverse_vjp(31.0, 2.0, torch.from_numpy(fb).cuda())
    ref = O.inverse_vjp(d, 31.0, 2.0, fb)
    for a, b in zip(got, ref):
        assert rel_err(host(a), b) <= FP64_REL_TOL
    k.close()


def test_rk4_step_vjp_matches_oracle(wv):
    c = config_from_case(golden_cases()["wave_16x16x9"])
    d = O.build_descriptor(c)
    rng = np.random.default_rng(6)
    A = [1e-2 * cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    yb = [cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    got = k.rk4_step_vjp(*(dev(x) for x in A), 40.0, 0.0, 30.0, *(dev(x) for x in yb))
    ref = O.rk4_step_vjp(d, *A, 40.0, 0.0, 30.0, yb)
    for a, b in zip(got, ref):
        assert rel_err(host(a), b) <= 1e-11
    k.close()


def test_checkpointed_adjoint_equals_chained_step_vjps(wv):
    import torch
    c = O.Config(Nx=32, Ny=32, Nz=17, Nj=10, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(7)
    A = O.spectrum_state(d, seed=2, urms=0.1)
    yb = [cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    dt, n = 300.0, 7
    got = k.rk4_adjoint(*(dev(x) for x in A), 0.0, 0.0, dt, n, 3, *(dev(x) for x in yb))
    # chain: forward states, then step VJPs backward
    states = []
    s = [dev(x) for x in A]
    t = 0.0
    for i in range(n):
        states.append((tuple(x.clone() for x in s), t))
        s = list(s)
        _, _, _, t = k.rk4(*s, t, 0.0, dt, 1)
    cur = [dev(x) for x in yb]
    for (st, ti) in reversed(states):
        cur = k.rk4_step_vjp(*st, ti, 0.0, dt, *cur)
    torch.cuda.synchronize()
    for a, b in zip(got, cur):
        assert np.array_equal(host(a), host(b))
    k.close()


def test_misfit_gradient_finite_differences(wv):
    """Final-state misfit gradient: J = 0.5 ||(u, v, eta)(T) - target||^2 after n RK4
    steps, adjoint gradient vs Richardson-extrapolated central differences along
    random directions (step 1e-6 x rms of the state)."""
    import torch
    c = O.Config(Nx=32, Ny=32, Nz=17, Nj=10, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    A = wv.synthetic_state(k, seed=11, urms=0.1)
    target_state = wv.synthetic_state(k, seed=12, urms=0.1)
    dt = wv.cfl_time_step(k, *A)
    n, K = 6, 2
    tgt = k.transformWaveVortexToUVWEta(n * dt, 0.0, *target_state)
    mask = np.array([1.0, 1.0, 0.0, 1.0])[:, None, None, None]

    def J(state):
        s = [dev(x) for x in state]
        _, _, _, tT = k.rk4(*s, 0.0, 0.0, dt, n)
        f = k.transformWaveVortexToUVWEta(tT, 0.0, *(host(x) for x in s))
        r = (f - tgt) * mask
        return 0.5 * float(np.sum(r * r)), [host(x) for x in s], tT

    J0, yT, tT = J(A)
    f = k.transformWaveVortexToUVWEta(tT, 0.0, *yT)
    fb = torch.from_numpy(np.ascontiguousarray((f - tgt) * mask)).cuda()
    ybT = k.inverse_vjp(tT, 0.0, fb)
    grad = k.rk4_adjoint(*(dev(x) for x in A), 0.0, 0.0, dt, n, K, *ybT)
    grad = [host(x) for x in grad]
    rms = float(np.sqrt(np.mean(np.concatenate([np.abs(x).ravel() ** 2 for x in A]))))
    rng = np.random.default_rng(8)
    for _ in range(4):
        direction = [cplx(rng, A[0].shape) for _ in range(3)]
        def dJ(eps):
            Jp = J([A[i] + eps * direction[i] for i in range(3)])[0]
            Jm = J([A[i] - eps * direction[i] for i in range(3)])[0]
            return (Jp - Jm) / (2 * eps)
        h = 1e-6 * rms
        fd = (4.0 * dJ(h / 2) - dJ(h)) / 3.0
        adj = inner(grad, direction)
        assert abs(fd - adj) <= 1e-5 * abs(adj), (fd, adj)
    k.close()


@pytest.mark.parametrize("Nx,Nz,hydro", [(64, 33, False), (128, 65, False), (256, 129, False), (128, 65, True), (96, 49, False)])
def test_mixed_adjoint_close_to_fp64(wv, Nx, Nz, hydro):
    """Mixed-precision VJP against the FP64 VJP (same state and cotangent); the
    mixed x pass adjoint runs on the warp FFTs for Nx = 64 R and on the
    shared-memory kernel otherwise (Nx = 96)."""
    c = O.Config(Nx=Nx, Ny=Nx, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Nx, Lz=4000.0, latitude=33.0,
                 isHydrostatic=hydro)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(9)
    A = O.spectrum_state(d, seed=3, urms=0.1)
    Fb = [cplx(rng, (d.Nkl, c.Nj)) for _ in range(3)]
    k64 = wv.WVTransformConstantStratificationKernel(to_wv(wv, c), precision="fp64")
    k32 = wv.WVTransformConstantStratificationKernel(to_wv(wv, c), precision="mixed")
    a = k64.flux_vjp(0.0, 0.0, *(dev(x) for x in A), *(dev(x) for x in Fb))
    b = k32.flux_vjp(0.0, 0.0, *(dev(x) for x in A), *(dev(x) for x in Fb))
    errs = [rel_err(host(y), host(x)) for x, y in zip(a, b)]
    print(f"mixed vs fp64 flux VJP max-relative error (Apb, Amb, A0b) {Nx}x{Nx}x{Nz} hydro={hydro}:", errs)
    assert max(errs) <= 1e-3
    k64.close()
    k32.close()


def test_autograd_misfit_gradient(wv):
    """The final-state misfit written as a torch expression over the autograd
    wrappers (tests/_torch_adjoint.py) and differentiated with backward(): the
    gradient equals the direct adjoint call and central differences along
    random directions."""
    import torch
    from _torch_adjoint import RK4Steps, WaveVortexToUVWEta
    c = O.Config(Nx=32, Ny=32, Nz=17, Nj=10, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    A = wv.synthetic_state(k, seed=11, urms=0.1)
    target_state = wv.synthetic_state(k, seed=12, urms=0.1)
    dt = wv.cfl_time_step(k, *A)
    n, K = 6, 3
    tT = n * dt
    tgt = torch.from_numpy(k.transformWaveVortexToUVWEta(tT, 0.0, *target_state)).cuda()
    mask = torch.tensor([1.0, 1.0, 0.0, 1.0], dtype=torch.float64, device="cuda")[:, None, None, None]

    def misfit(y0):
        yT = RK4Steps.apply(*y0, k, 0.0, 0.0, dt, n, K)
        f = WaveVortexToUVWEta.apply(*yT, k, tT, 0.0)
        r = (f - tgt) * mask
        return 0.5 * (r * r).sum()

    y0 = [dev(x).requires_grad_(True) for x in A]
    J = misfit(y0)
    J.backward()
    grad = [host(x.grad) for x in y0]
    # the same gradient from the C entry points directly
    with torch.no_grad():
        yT = [dev(x) for x in A]
        k.rk4(*yT, 0.0, 0.0, dt, n)
        fb = ((k.transformWaveVortexToUVWEta(tT, 0.0, *yT) - tgt) * mask).contiguous()
        direct = [host(x) for x in k.rk4_adjoint(*(dev(x) for x in A), 0.0, 0.0, dt, n, K, *k.inverse_vjp(tT, 0.0, fb))]
    for a, b in zip(grad, direct):
        assert np.array_equal(a, b)
    rms = float(np.sqrt(np.mean(np.concatenate([np.abs(x).ravel() ** 2 for x in A]))))
    rng = np.random.default_rng(21)
    with torch.no_grad():
        for _ in range(3):
            direction = [cplx(rng, A[0].shape) for _ in range(3)]
            def dJ(eps):
                Jp = float(misfit([dev(A[i] + eps * direction[i]) for i in range(3)]))
                Jm = float(misfit([dev(A[i] - eps * direction[i]) for i in range(3)]))
                return (Jp - Jm) / (2 * eps)
            h = 1e-6 * rms
            fd = (4.0 * dJ(h / 2) - dJ(h)) / 3.0
            adj = inner(grad, direction)
            assert abs(fd - adj) <= 1e-5 * abs(adj), (fd, adj)
    k.close()

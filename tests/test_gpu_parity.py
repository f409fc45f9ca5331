"""Parity of the CUDA path (through the C ABI) against the reference's golden
vectors and the numpy oracle.  FP64 gate: 1e-12 relative, the reference's own
compiled-backend gate (WVCompiledConstantStratificationBackend.m:152)."""
import numpy as np
import pytest

import wv_oracle as O
from _cases import FP64_REL_TOL, config_from_case, golden_cases, load_golden, parity_tolerance, rel_err, state_components_close

pytestmark = pytest.mark.gpu

CASES = golden_cases()


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def to_wv(wvgpu, c):
    return wvgpu.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                               planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                               isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


@pytest.fixture(scope="module", params=sorted(CASES))
def gcase(request, wv):
    name = request.param
    cf = CASES[name]
    c = config_from_case(cf)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    yield name, cf, k, load_golden(name)
    k.close()


def test_flux_matches_reference(gcase):
    name, cf, k, g = gcase
    F = k.nonlinearFlux(float(g["t"]), float(g["t0"]), g["Ap"], g["Am"], g["A0"])
    for got, key in zip(F, ("Fp", "Fm", "F0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, (name, key, rel_err(got, g[key]))


def test_scheduled_rhs_matches_reference(gcase):
    name, cf, k, g = gcase
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    try:
        R = k.evaluateRightHandSide(float(g["t"]), float(g["t0"]), g["Ap"], g["Am"], g["A0"])
    finally:
        k.set_forcing(nonlinear=True, adaptive_damping=False)
    for got, key in zip(R, ("Rp", "Rm", "R0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, (name, key, rel_err(got, g[key]))


def test_forward_matches_reference(gcase):
    name, cf, k, g = gcase
    fwd = k.transformUVEtaToWaveVortex if cf["isHydrostatic"] else k.transformUVWEtaToWaveVortex
    B = fwd(g["fields"], float(g["t"]), float(g["t0"]))
    for got, key in zip(B, ("Bp", "Bm", "B0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, (name, key, rel_err(got, g[key]))


def test_inverse_matches_reference(gcase):
    name, cf, k, g = gcase
    f = k.transformWaveVortexToUVWEta(float(g["t"]), float(g["t0"]), g["Ap"], g["Am"], g["A0"])
    assert rel_err(f, g["inverse"]) <= FP64_REL_TOL, (name, rel_err(f, g["inverse"]))


def test_rk4_matches_reference(gcase):
    name, cf, k, g = gcase
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    try:
        K = k.rk4(g["rk_Ap"], g["rk_Am"], g["rk_A0"], float(g["rk_t"]), float(g["rk_t0"]), float(g["rk_dt"]),
                  int(g["rk_steps"]))
    finally:
        k.set_forcing(nonlinear=True, adaptive_damping=False)
    assert not state_components_close(K[:3], g, ("Kp", "Km", "K0"), FP64_REL_TOL), name
    assert K[3] == float(g["rk_tout"])


def test_device_entries_match_host_entries(gcase):
    import torch
    name, cf, k, g = gcase
    t, t0 = float(g["t"]), float(g["t0"])
    Fh = k.nonlinearFlux(t, t0, g["Ap"], g["Am"], g["A0"])
    dev = [torch.from_numpy(np.ascontiguousarray(g[n])).cuda() for n in ("Ap", "Am", "A0")]
    Fd = k.nonlinearFlux(t, t0, *dev)
    torch.cuda.synchronize()
    for a, b in zip(Fh, Fd):
        assert np.array_equal(a, b.cpu().numpy())


def test_zero_state_gives_exactly_zero_flux(wv):
    """TestWVKernelContract.cpp:395-414."""
    c = config_from_case(CASES["odd_15x13x9"])
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    d = O.build_descriptor(c)
    z = np.zeros((d.Nkl, c.Nj), np.complex128)
    F = k.nonlinearFlux(3.0, 1.0, z, z, z)
    for x in F:
        assert np.all(x == 0) and np.all(np.isfinite(x))
    k.close()


def _mid_case(Nx, Ny, Nz, hydro=False, antialias=True, lat=33.0, L=400e3):
    return O.Config(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=L, Ly=L * Ny / Nx, Lz=4000.0, latitude=lat,
                    isHydrostatic=hydro, shouldAntialias=antialias)


@pytest.mark.parametrize("shape,hydro", [((64, 64, 33), False), ((48, 40, 17), True), ((96, 72, 25), False),
                                         ((30, 27, 11), False)])
def test_flux_matches_oracle_mid_sizes(wv, shape, hydro):
    # Representable random flow at 0.1 m/s rms, as the reference's self-test uses
    # (initWithRandomFlow, wvCompiledBackendBuild.m:356-398); arbitrary
    # coefficients are covered by the golden cases.
    c = _mid_case(*shape, hydro=hydro)
    d = O.build_descriptor(c)
    Ap, Am, A0 = O.spectrum_state(d, seed=7, urms=0.1)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    F = k.nonlinearFlux(1234.5, 10.0, Ap, Am, A0)
    R, floors = O.noise_floor(O.nonlinear_flux, d, Ap, Am, A0, 1234.5, 10.0)
    for a, b, fl in zip(F, R, floors):
        assert rel_err(a, b) <= parity_tolerance(fl), (rel_err(a, b), fl)
    k.close()


@pytest.mark.parametrize("shape,hydro", [((64, 64, 33), False), ((48, 40, 17), True)])
def test_round_trip_identity(wv, shape, hydro):
    """inverse -> forward reproduces representable coefficients, at the
    reference's round-trip tolerance 5e-10 (TestCoreTransformInvariants.m:79-85;
    the separation of Ap from Am in near-inertial low-Kh modes is ill-conditioned
    even in exact FP64 evaluation order)."""
    c = _mid_case(*shape, hydro=hydro)
    d = O.build_descriptor(c)
    A = O.random_state(d, seed=3, scale=1e-3)
    f = O.inverse_uvweta(d, *A, 0.0, 0.0)
    A = O.forward(d, f[[0, 1, 3]] if hydro else f, 0.0, 0.0)  # representable flat-spectrum flow
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    f = k.transformWaveVortexToUVWEta(50.0, 0.0, *A)
    fo = O.inverse_uvweta(d, *A, 50.0, 0.0)
    assert rel_err(f, fo) <= FP64_REL_TOL
    fwd = k.transformUVEtaToWaveVortex if hydro else k.transformUVWEtaToWaveVortex
    B = fwd(f[[0, 1, 3]] if hydro else f, 50.0, 0.0)
    Bo = O.forward(d, fo[[0, 1, 3]] if hydro else fo, 50.0, 0.0)
    for a, b, o in zip(B, A, Bo):
        # the oracle's own FP64 round trip sets the conditioning of this state
        assert rel_err(a, b) <= max(5e-10, 3.0 * rel_err(o, b)), (rel_err(a, b), rel_err(o, b))
    k.close()


def test_transforms_match_oracle_steep_spectrum(wv):
    """192x192x97 (radix-3 FFTs), benchmark spectrum: inverse at 1e-12; forward
    against the oracle's forward within the measured FP64 noise floor."""
    c = _mid_case(192, 192, 97)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=3, urms=0.1)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    f = k.transformWaveVortexToUVWEta(50.0, 0.0, *A)
    fo = O.inverse_uvweta(d, *A, 50.0, 0.0)
    assert rel_err(f, fo) <= FP64_REL_TOL
    B = k.transformUVWEtaToWaveVortex(fo, 50.0, 0.0)
    R, floors = O.noise_floor(O.forward, d, fo, 50.0, 0.0)
    for a, b, fl in zip(B, R, floors):
        assert rel_err(a, b) <= parity_tolerance(fl), (rel_err(a, b), fl)
    k.close()


def test_full_size_flux_and_energy_conservation(wv):
    """256x256x129 (the benchmark grid): flux vs oracle at 1e-12 and the inviscid
    energy flux sum (energyFluxFromNonlinearFlux.m:37-44) vanishing."""
    c = O.Config(Nx=256, Ny=256, Nz=129, Nj=85, Lx=800e3, Ly=800e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    Ap, Am, A0 = O.spectrum_state(d, seed=1, urms=0.1)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    F = k.nonlinearFlux(0.0, 0.0, Ap, Am, A0)
    R, floors = O.noise_floor(O.nonlinear_flux, d, Ap, Am, A0, 0.0, 0.0)
    for a, b, fl in zip(F, R, floors):
        assert rel_err(a, b) <= parity_tolerance(fl), (rel_err(a, b), fl)
    Ep, Em, E0 = O.energy_flux(d, Ap, Am, A0, *F)
    total = np.sum(Ep) + np.sum(Em) + np.sum(E0)
    scale = np.sum(np.abs(Ep)) + np.sum(np.abs(Em)) + np.sum(np.abs(E0))
    # Tolerance: quadratic conservation to rounding; 1e-11 relative at this size.
    assert abs(total) / scale <= 1e-11
    k.close()


def test_gpu_synthetic_state_matches_oracle(wv):
    """The benchmark's GPU-built synthetic state equals the oracle's construction."""
    c = _mid_case(64, 64, 33)
    d = O.build_descriptor(c)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    A = wv.synthetic_state(k, seed=5, urms=0.1)
    B = O.spectrum_state(d, seed=5, urms=0.1)
    # Same flow: compare the physical fields (coefficients of ill-conditioned
    # near-inertial modes carry the round trip's FP64 noise).
    assert rel_err(O.inverse_uvweta(d, *A, 0.0, 0.0), O.inverse_uvweta(d, *B, 0.0, 0.0)) <= 1e-10
    assert abs(wv.cfl_time_step(k, *A) - O.cfl_time_step(d, *B)) <= 1e-9 * O.cfl_time_step(d, *B)
    k.close()


def test_stage_instrumentation(wv):
    c = _mid_case(64, 64, 33)
    d = O.build_descriptor(c)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    Ap, Am, A0 = O.spectrum_state(d, seed=2, urms=0.1)
    k.setStageInstrumentation(True)
    F1 = k.nonlinearFlux(0.0, 0.0, Ap, Am, A0)
    st = k.stage_times()
    k.setStageInstrumentation(False)
    F2 = k.nonlinearFlux(0.0, 0.0, Ap, Am, A0)
    assert st["fluxes"] == 1 and all(st[n] > 0 for n in st if n.endswith("_ms"))
    for a, b in zip(F1, F2):
        assert np.array_equal(a, b)
    k.close()


def test_single_wave_16x16x9_to_t600_matches_reference(wv):
    """16x16x9 end to end: single internal wave (kMode=1, lMode=0, j=1,
    u = 0.05 m/s) under {nonlinear advection, adaptive damping}, 60 RK4 steps of
    10 s to t = 600 s, field by field against the reference FP64 path (its own
    run, tests/golden/wave_16x16x9_t600.npz)."""
    import os
    c = config_from_case(golden_cases()["wave_16x16x9"])
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "wave_16x16x9_t600.npz"))
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    k.set_forcing(nonlinear=True, adaptive_damping=True)
    Ap, Am, A0, t = k.rk4(g["Ap"], g["Am"], g["A0"], 0.0, 0.0, float(g["dt"]), int(g["steps"]))
    assert t == float(g["t"])
    assert not state_components_close((Ap, Am, A0), g, ("Kp", "Km", "K0"), FP64_REL_TOL)
    assert rel_err(k.transformWaveVortexToUVWEta(t, 0.0, Ap, Am, A0), g["fields"]) <= FP64_REL_TOL
    k.close()

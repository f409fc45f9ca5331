"""nonlinearFluxWithAdvectionFields / nonlinearFluxUsingAdvectionFields and
transformWaveVortexToUVW through the C ABI against the reference's own outputs
(golden fixtures) and the oracle at larger sizes."""
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


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_advection_field_entries_match_reference(wv, name):
    import torch
    c = config_from_case(golden_cases()[name])
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    args = (float(g["t"]), float(g["t0"]), g["Ap"], g["Am"], g["A0"])
    F, adv = k.nonlinearFluxWithAdvectionFields(*args)
    for a, b in zip(F, (g["with_Fp"], g["with_Fm"], g["with_F0"])):
        assert rel_err(a, b) <= FP64_REL_TOL
    assert rel_err(adv, g["with_fields"]) <= FP64_REL_TOL
    F = k.nonlinearFluxUsingAdvectionFields(*args, g["given_fields"])
    for a, b in zip(F, (g["using_Fp"], g["using_Fm"], g["using_F0"])):
        assert rel_err(a, b) <= FP64_REL_TOL
    assert rel_err(k.transformWaveVortexToUVW(*args), g["uvw"]) <= FP64_REL_TOL
    # device-pointer forms give the same numbers
    dev = [torch.from_numpy(np.ascontiguousarray(g[n])).cuda() for n in ("Ap", "Am", "A0")]
    Fd, advd = k.nonlinearFluxWithAdvectionFields(args[0], args[1], *dev)
    assert np.array_equal(advd.cpu().numpy(), adv)
    Fu = k.nonlinearFluxUsingAdvectionFields(args[0], args[1], *dev, torch.from_numpy(g["given_fields"]).cuda())
    for a, b in zip(Fu, (g["using_Fp"], g["using_Fm"], g["using_F0"])):
        assert rel_err(a.cpu().numpy(), b) <= FP64_REL_TOL
    k.close()


@pytest.mark.parametrize("shape,precision", [((64, 64, 33), "fp64"), ((64, 64, 33), "mixed"), ((48, 40, 25), "fp64")])
def test_using_own_advection_fields_equals_flux(wv, shape, precision):
    """The flux advected by the fields the flux itself returns is the flux (FP64:
    to rounding; mixed: the fields pass through double, so to FP32 rounding)."""
    import torch
    Nx, Ny, Nz = shape
    cfg = wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0,
                           latitude=33.0)
    k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
    A = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in wv.synthetic_state(k, seed=3, urms=0.1)]
    F0 = [x.cpu().numpy() for x in k.nonlinearFlux(50.0, 0.0, *A)]
    F1, adv = k.nonlinearFluxWithAdvectionFields(50.0, 0.0, *A)
    F2 = k.nonlinearFluxUsingAdvectionFields(50.0, 0.0, *A, adv)
    for a, b in zip(F1, F0):
        assert np.array_equal(a.cpu().numpy(), b)
    tol = 1e-13 if precision == "fp64" else 1e-5
    for a, b in zip(F2, F0):
        assert rel_err(a.cpu().numpy(), b) <= tol
    uvw = k.transformWaveVortexToUVW(50.0, 0.0, *A).cpu().numpy()
    assert rel_err(adv.cpu().numpy(), uvw) <= (1e-13 if precision == "fp64" else 1e-5)
    k.close()


def test_advection_fields_overlap_rejected(wv):
    import torch
    c = config_from_case(golden_cases()["wave_16x16x9"])
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    g = load_golden("wave_16x16x9")
    buf = torch.zeros(3 * c.Nx * c.Ny * c.Nz * 2, dtype=torch.float64, device="cuda")
    A = [torch.from_numpy(np.ascontiguousarray(g[n])).cuda() for n in ("Ap", "Am", "A0")]
    # a flux output inside the fields buffer
    Fp = torch.view_as_complex(buf[: 2 * A[0].numel()].view(-1, 2)).view(A[0].shape)
    import ctypes
    rc = k._lib.wv_nonlinear_flux_with_advection_fields_device(
        k._h, 0.0, 0.0, A[0].data_ptr(), A[1].data_ptr(), A[2].data_ptr(), Fp.data_ptr(),
        torch.empty_like(A[0]).data_ptr(), torch.empty_like(A[0]).data_ptr(), buf.data_ptr(), k._stream())
    assert rc == 4
    k.close()


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_field_derivatives_match_reference(wv, name):
    cf = golden_cases()[name]
    c = config_from_case(cf)
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    for q in ((0, 1, 3) if cf["isHydrostatic"] else (0, 1, 2, 3)):
        got = k.transformStateFieldDerivatives(float(g["t"]), float(g["t0"]), g["Ap"], g["Am"], g["A0"], q)
        assert rel_err(got, g[f"deriv_{q}"]) <= FP64_REL_TOL, q
    k.close()


@pytest.mark.parametrize("name", sorted(golden_cases()))
@pytest.mark.parametrize("antialias", [False, True])
def test_fgrid_scalar_advection_matches_reference(wv, name, antialias):
    c = config_from_case(golden_cases()[name])
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    got = k.advectFGridScalar(g["scalar"], g["given_fields"], antialias)
    ref = g["scalar_rhs_aa"] if antialias else g["scalar_rhs"]
    assert rel_err(got, ref) <= FP64_REL_TOL
    k.close()


@pytest.mark.parametrize("shape", [(64, 64, 33), (48, 40, 25), (96, 80, 49)])
def test_fgrid_scalar_advection_vs_oracle_midsize(wv, shape):
    """Larger grids against the oracle (noise-floor gated), device-pointer form."""
    import torch
    Nx, Ny, Nz = shape
    c = O.Config(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(17)
    scalar = rng.standard_normal((Nz, Ny, Nx))
    adv = rng.standard_normal((3, Nz, Ny, Nx)) * 0.1
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    for aa in (False, True):
        got = k.advectFGridScalar(torch.from_numpy(scalar).cuda(), torch.from_numpy(adv).cuda(), aa).cpu().numpy()
        ref, floors = O.noise_floor(lambda *a: (O.advect_fgrid_scalar(*a),), d, scalar, adv, aa)
        assert rel_err(got, ref[0]) <= parity_tolerance(floors[0]), (aa, rel_err(got, ref[0]), floors[0])
    k.close()


def test_field_derivatives_vs_oracle_midsize(wv):
    import torch
    c = O.Config(Nx=64, Ny=64, Nz=33, Nj=21, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=5, urms=0.1)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    for q in range(4):
        got = k.transformStateFieldDerivatives(300.0, 0.0, *(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A), q)
        ref, floors = O.noise_floor(lambda *a: (O.derivative_fields(*a),), d, *A, 300.0, 0.0, q)
        assert rel_err(got.cpu().numpy(), ref[0]) <= parity_tolerance(floors[0]), q
    k.close()


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_family_derivatives_match_reference(wv, name):
    import torch
    c = config_from_case(golden_cases()[name])
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    assert rel_err(k.transformToSpatialDomainWithFAllDerivatives(g["Apm"], g["A0"]), g["fall"]) <= FP64_REL_TOL
    assert rel_err(k.transformToSpatialDomainWithGAllDerivatives(g["Apm"], g["A0"]), g["gall"]) <= FP64_REL_TOL
    dev = [torch.from_numpy(np.ascontiguousarray(g[n])).cuda() for n in ("Apm", "A0")]
    assert rel_err(k.transformToSpatialDomainWithFAllDerivatives(*dev).cpu().numpy(), g["fall"]) <= FP64_REL_TOL
    k.close()


def test_family_derivatives_vs_oracle_midsize(wv):
    c = O.Config(Nx=64, Ny=48, Nz=33, Nj=21, Lx=400e3, Ly=300e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(23)
    Apm = rng.standard_normal((d.Nkl, c.Nj)) + 1j * rng.standard_normal((d.Nkl, c.Nj))
    A0 = rng.standard_normal((d.Nkl, c.Nj)) + 1j * rng.standard_normal((d.Nkl, c.Nj))
    k = wv.WVTransformConstantStratificationKernel(to_wv(wv, c))
    for ff in (True, False):
        got = k._family(ff, Apm, A0)
        ref, floors = O.noise_floor(lambda *a: (O.family_derivatives(*a),), d, Apm, A0, ff)
        assert rel_err(got, ref[0]) <= parity_tolerance(floors[0]), ff
    k.close()

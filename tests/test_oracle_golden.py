"""Pins the numpy oracle against golden vectors produced by the reference's own
C++ kernel (CompiledKernel + PortableRuntime, exact direct-DFT engine)."""
import numpy as np
import pytest

import wv_oracle as O
from _cases import FP64_REL_TOL, config_from_case, golden_cases, load_golden, rel_err

CASES = golden_cases()


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    name = request.param
    cf = CASES[name]
    desc = O.build_descriptor(config_from_case(cf))
    return name, cf, desc, load_golden(name)


def test_descriptor_ordering_and_arrays_bitwise(case):
    name, cf, d, g = case
    assert np.array_equal(d.kMode, g["desc_kMode"])
    assert np.array_equal(d.lMode, g["desc_lMode"])
    assert np.array_equal(d.storageRow, g["desc_storageRow"])
    assert np.array_equal(d.conjugated, g["desc_conjugated"])
    # Mode-set construction restates WVKernelTypes.cpp:119-330 operation for operation.
    assert np.array_equal(d.arrays["omega"].ravel(), g["desc_omega"])
    assert np.array_equal(d.arrays["fWaveScale"].ravel(), g["desc_fWaveScale"])
    assert np.array_equal(d.arrays["UAp"].ravel(), g["desc_UApField"])
    assert np.array_equal(d.arrays["WAp"].ravel(), g["desc_WApField"])
    assert np.array_equal(d.arrays["A0FromVorticity"].ravel(), g["desc_A0FromVorticity"])
    assert np.array_equal(d.arrays["A0FromBuoyancy"].ravel(), g["desc_A0FromBuoyancy"])
    assert np.array_equal(d.arrays["NA0"].ravel(), g["desc_NA0Field"])
    assert np.array_equal(d.arrays["ApmN"].ravel(), g["desc_ApmNProjection"])


def test_nonlinear_flux(case):
    name, cf, d, g = case
    F = O.nonlinear_flux(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]))
    for got, key in zip(F, ("Fp", "Fm", "F0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, key


def test_scheduled_rhs(case):
    name, cf, d, g = case
    damp = O.adaptive_damping_operator(d) if cf["damping"] else None
    R = O.rhs(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]), damp)
    for got, key in zip(R, ("Rp", "Rm", "R0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, key


def test_forward_transform(case):
    name, cf, d, g = case
    B = O.forward(d, g["fields"], float(g["t"]), float(g["t0"]))
    for got, key in zip(B, ("Bp", "Bm", "B0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, key


def test_inverse_transform(case):
    name, cf, d, g = case
    inv = O.inverse_uvweta(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]))
    assert rel_err(inv, g["inverse"]) <= FP64_REL_TOL


def test_fixed_rk4(case):
    name, cf, d, g = case
    damp = O.adaptive_damping_operator(d) if cf["damping"] else None
    K = O.rk4(d, g["rk_Ap"], g["rk_Am"], g["rk_A0"], float(g["rk_t"]), float(g["rk_t0"]), float(g["rk_dt"]),
              int(g["rk_steps"]), damp)
    for got, key in zip(K[:3], ("Kp", "Km", "K0")):
        assert rel_err(got, g[key]) <= FP64_REL_TOL, key
    assert K[3] == float(g["rk_tout"])


def test_zero_state_gives_exactly_zero_flux():
    """TestWVKernelContract.cpp:395-414: zero state -> bit-exact zero flux."""
    cf = CASES["odd_15x13x9"]
    d = O.build_descriptor(config_from_case(cf))
    z = np.zeros((d.Nkl, d.c.Nj), np.complex128)
    F = O.nonlinear_flux(d, z, z, z, 3.0, 1.0)
    for x in F:
        assert np.all(x == 0)


def test_invalid_configuration_rejected():
    cf = dict(CASES["odd_15x13x9"])
    c = config_from_case(cf)
    c.Nj = c.Nz
    with pytest.raises(O.OracleError) as e:
        O.build_descriptor(c)
    assert e.value.code == O.INVALID_CONFIGURATION


# ---- advection-field entry points, UVW inverse, state-field derivatives and
#      F-grid scalar advection against the reference's own outputs

@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_flux_with_and_using_advection_fields(name):
    c = config_from_case(golden_cases()[name])
    d = O.build_descriptor(c)
    g = load_golden(name)
    args = (g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]))
    (Fp, Fm, F0), adv = O.flux_with_advection(d, *args)
    for a, b in zip((Fp, Fm, F0), (g["with_Fp"], g["with_Fm"], g["with_F0"])):
        assert rel_err(a, b) <= 1e-12
    assert rel_err(adv, g["with_fields"]) <= 1e-12
    F = O.nonlinear_flux(d, *args, advection=g["given_fields"])
    for a, b in zip(F, (g["using_Fp"], g["using_Fm"], g["using_F0"])):
        assert rel_err(a, b) <= 1e-12
    assert rel_err(O.inverse_uvw(d, *args), g["uvw"]) <= 1e-12


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_field_derivatives(name):
    cf = golden_cases()[name]
    c = config_from_case(cf)
    d = O.build_descriptor(c)
    g = load_golden(name)
    for q in ((0, 1, 3) if cf["isHydrostatic"] else (0, 1, 2, 3)):
        got = O.derivative_fields(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]), q)
        assert rel_err(got, g[f"deriv_{q}"]) <= 1e-12, q


@pytest.mark.parametrize("name", sorted(golden_cases()))
@pytest.mark.parametrize("antialias", [False, True])
def test_oracle_fgrid_scalar_advection(name, antialias):
    c = config_from_case(golden_cases()[name])
    d = O.build_descriptor(c)
    g = load_golden(name)
    got = O.advect_fgrid_scalar(d, g["scalar"], g["given_fields"], antialias)
    ref = g["scalar_rhs_aa"] if antialias else g["scalar_rhs"]
    assert rel_err(got, ref) <= 1e-12


@pytest.mark.parametrize("name", sorted(golden_cases()))
def test_oracle_family_derivatives(name):
    c = config_from_case(golden_cases()[name])
    d = O.build_descriptor(c)
    g = load_golden(name)
    assert rel_err(O.family_derivatives(d, g["Apm"], g["A0"], True), g["fall"]) <= 1e-12
    assert rel_err(O.family_derivatives(d, g["Apm"], g["A0"], False), g["gall"]) <= 1e-12


def test_oracle_single_wave_to_t600():
    """16x16x9: single internal wave under {nonlinear advection, adaptive damping},
    60 RK4 steps of 10 s, against the reference's own run (coefficients and fields)."""
    c = config_from_case(golden_cases()["wave_16x16x9"])
    d = O.build_descriptor(c)
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "wave_16x16x9_t600.npz"))
    damp = O.adaptive_damping_operator(d)
    Ap, Am, A0, t = O.rk4(d, g["Ap"], g["Am"], g["A0"], 0.0, 0.0, float(g["dt"]), int(g["steps"]), damping=damp)
    assert t == float(g["t"])
    for a, b in zip((Ap, Am, A0), (g["Kp"], g["Km"], g["K0"])):
        assert rel_err(a, b) <= 1e-12
    assert rel_err(O.inverse_uvweta(d, Ap, Am, A0, t, 0.0), g["fields"]) <= 1e-12

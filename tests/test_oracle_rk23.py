"""Pins the oracle's adaptive RK23 (WVAdaptiveRK23 restated) against the
reference's own known answers (TestWVUnifiedIntegration.cpp:366-478) and
against runs of the reference integrator on the wave-vortex system
(tests/golden/rk23.npz)."""
import math

import numpy as np
import pytest

import wv_oracle as O
from _cases import RK23_RUNS, config_from_case, rk23_run


def test_matlab_ode23_parity_linear_system():
    """TestWVUnifiedIntegration.cpp:437-478: dy/dt = -y from (1, 0.5) on [0, 1],
    rtol 1e-8, absolute tolerance 1e-10, maximum step 0.5."""
    y = [np.array([[1.0 + 0.5j]]) for _ in range(3)]
    rk = O.RK23(lambda y, t: [-v for v in y], [np.full((1, 1), 1e-10)] * 3, rtol=1e-8, max_step=0.5)
    yy, t = rk.advance_to_time(y, 0.0, 1.0, 0.5)
    assert t == 1.0
    assert (rk.accepted_steps, rk.rejected_steps, rk.evaluations) == (159, 6, 496)
    assert len(rk.diagnostics) == 159
    assert abs(rk.diagnostics[0][1] - 0.0078125) < 1e-15
    assert abs(yy[0][0, 0].real - 0.36787943731476008) < 1e-14
    assert abs(yy[0][0, 0].imag - 0.18393971865738004) < 1e-14


def test_controller_work_zero_derivative():
    """TestWVUnifiedIntegration.cpp:402-435."""
    y = [np.zeros((3, 2), complex) for _ in range(3)]
    rk = O.RK23(lambda y, t: [0 * v for v in y], [np.full((3, 2), 1e-10)] * 3, max_step=0.1)
    rk.advance_to_time(y, 0.0, 1.0, 0.5)
    assert (rk.accepted_steps, rk.rejected_steps, rk.evaluations) == (10, 0, 31)
    assert all(abs(d[1] - 0.1) < 1e-14 and d[4] == 0 and d[2] == 0.0 for d in rk.diagnostics)
    assert not rk.diagnostics[0][6] and rk.diagnostics[-1][6]


def test_no_growth_after_rejection_and_dense_output():
    """TestWVUnifiedIntegration.cpp:366-390."""
    y = [np.array([[1.0 + 0j]]) for _ in range(3)]
    rk = O.RK23(lambda y, t: [-v for v in y], [np.full((1, 1), 1e-10)] * 3, rtol=1e-8, max_factor=2.0)
    _, t = rk.step(y, 0.0, 0.5)
    assert rk.rejected_steps > 0
    ti, tf, _ = rk.accepted
    assert abs(rk.next_step - (tf - ti)) < 1e-15
    mid = 0.5 * (ti + tf)
    assert abs(rk.dense_output(mid)[0][0, 0].real - math.exp(-mid)) < 1e-6


def test_errors():
    rk = O.RK23(lambda y, t: [-v for v in y], [np.full((1, 1), 1e-10)] * 3)
    with pytest.raises(O.OracleError) as e:
        rk.dense_output(0.0)
    assert e.value.code == 10
    with pytest.raises(O.OracleError) as e:
        rk.advance_to_time([np.ones((1, 1), complex)] * 3, 1.0, 0.5, 0.1)
    assert e.value.code == 1
    with pytest.raises(O.OracleError) as e:
        rk.step([np.ones((1, 1), complex)] * 3, 0.0, -1.0)
    assert e.value.code == 1


@pytest.mark.parametrize("key", sorted(RK23_RUNS))
def test_wave_vortex_run_matches_reference_integrator(key):
    """The oracle's RK23 on the oracle's right-hand side reproduces the
    reference integrator's run: the same accepted/rejected/evaluation counts,
    the tolerance audit hashes bit for bit, step sizes and normalized errors
    to FP64 noise (the error norm divides small differences), the end state
    and the dense output at the FP64 parity gate."""
    cf, options, ref = rk23_run(key)
    d = O.build_descriptor(config_from_case(cf))
    damping = O.adaptive_damping_operator(d) if cf["damping"] else None
    Ap, Am, A0, t, rk = O.rk23_advance(d, ref["Ap"], ref["Am"], ref["A0"], ref["t"], ref["t0"], ref["final"],
                                       ref["initial"], damping=damping, **options)
    assert t == ref["tout"]
    assert [rk.accepted_steps, rk.rejected_steps, rk.evaluations, rk.fsal_reuses] == ref["counts"].tolist()
    wave, vortex = O.rk23_tolerances(d, options["atol_scale"])
    total, per = O.rk23_tolerance_hash([wave, wave, vortex])
    assert [total] + per == [int(v) for v in ref["hashes"]]
    diag = np.array([x[:6] for x in rk.diagnostics])
    assert diag.shape == ref["diag"][:, :6].shape
    assert np.array_equal(diag[:, 4], ref["diag"][:, 4]) and np.array_equal(diag[:, 5], ref["diag"][:, 5])
    assert np.array_equal(np.array([x[6] for x in rk.diagnostics], float), ref["diag"][:, 6])
    assert np.max(np.abs(diag[:, 1] - ref["diag"][:, 1]) / ref["diag"][:, 1]) < 1e-6
    assert abs(rk.next_step - ref["next"]) / ref["next"] < 1e-6
    for got, want in zip((Ap, Am, A0), (ref["Kp"], ref["Km"], ref["K0"])):
        if np.any(want):
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-11
    dense = rk.dense_output(ref["dense_time"])
    for got, want in zip(dense, ref["dense"]):
        if np.any(want):
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-11


@pytest.mark.parametrize("key", ["odd", "hd"])
def test_rk4_advance_and_dense_output_match_reference(key):
    """WVFixedStepRK4::advanceToTime with a final partial step and the retained
    cubic Hermite dense output, against the reference integrator."""
    from _cases import rk4_dense_run
    cf, g = rk4_dense_run(key)
    d = O.build_descriptor(config_from_case(cf))
    damping = O.adaptive_damping_operator(d) if bool(g["damping"]) else None
    Ap, Am, A0, t, dense = O.rk4_advance_to_time(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]),
                                                 float(g["final"]), float(g["dt"]), damping)
    assert t == float(g["tout"])
    assert (dense[0], dense[1]) == tuple(g["interval"].tolist())
    for got, want in zip((Ap, Am, A0), (g["Kp"], g["Km"], g["K0"])):
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12
    out = O.rk4_dense_output(dense, float(g["dense_time"]))
    for got, want in zip(out, g["dense"]):
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12

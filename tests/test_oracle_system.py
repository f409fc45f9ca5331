"""Pins the oracle's integration system with integrated observers (particle
groups with linear and spline velocity sampling, F-grid tracers) against the
reference's WVConstantStratificationIntegrationSystem
(PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:295-400):
one right-hand side, RK4 steps and an adaptive RK23 interval per fixture run
(tests/golden/system.npz)."""
import numpy as np
import pytest

import wv_oracle as O
from _cases import config_from_case, rel_err, split_extra, system_observers, system_run

RUNS = ["obs", "hd"]


def _setup(key):
    cf, run, g = system_run(key)
    d = O.build_descriptor(config_from_case(cf))
    groups, tracers = system_observers(run)
    damping = O.adaptive_damping_operator(d) if run["schedule"] == 1 else None
    y = [g["Ap"], g["Am"], g["A0"]] + split_extra(d, groups, tracers, g["extra"])
    return d, run, g, groups, tracers, damping, y


@pytest.mark.parametrize("key", RUNS)
def test_system_rhs_matches_reference(key):
    d, run, g, groups, tracers, damping, y = _setup(key)
    out = O.system_rhs(d, y, float(g["t"]), float(g["t0"]), groups, tracers, damping)
    for got, want in zip(out[:3], (g["Fp"], g["Fm"], g["F0"])):
        assert rel_err(got, want) <= 1e-12
    want = split_extra(d, groups, tracers, g["rhs_extra"])
    assert len(want) == len(out) - 3
    for i, (got, w) in enumerate(zip(out[3:], want)):
        assert rel_err(got, w) <= 1e-11, (key, i, rel_err(got, w))


@pytest.mark.parametrize("key", RUNS)
def test_system_rk4_matches_reference(key):
    d, run, g, groups, tracers, damping, y = _setup(key)
    yk, t = O.system_rk4(d, y, float(g["t"]), float(g["t0"]), float(g["dt"]), int(g["steps"]), groups, tracers, damping)
    assert t == float(g["k_t"])
    for got, want in zip(yk[:3], (g["Kp"], g["Km"], g["K0"])):
        assert rel_err(got, want) <= 1e-12
    for got, want in zip(yk[3:], split_extra(d, groups, tracers, g["k_extra"])):
        assert rel_err(got, want) <= 1e-12


@pytest.mark.parametrize("key", RUNS)
def test_system_rk23_matches_reference(key):
    d, run, g, groups, tracers, damping, y = _setup(key)
    o = g["rk23_opts"]
    yr, t, rk = O.system_rk23_advance(d, y, float(g["t"]), float(g["t0"]), float(g["rk23_final"]),
                                      float(g["rk23_initial"]), groups, tracers, damping, rtol=float(o[0]),
                                      atol_scale=float(o[1]), safety=float(o[2]), floor=float(o[3]),
                                      max_factor=float(o[4]), max_step=float(o[5]))
    assert t == float(g["r_t"])
    assert [rk.accepted_steps, rk.rejected_steps, rk.evaluations, rk.fsal_reuses] == g["r_counts"].tolist()
    steps = np.array([x[1] for x in rk.diagnostics])
    assert np.max(np.abs(steps - g["r_steps"]) / g["r_steps"]) < 1e-6
    for got, want in zip(yr[:3], (g["Rp"], g["Rm"], g["R0"])):
        assert rel_err(got, want) <= 1e-11
    for got, want in zip(yr[3:], split_extra(d, groups, tracers, g["r_extra"])):
        assert rel_err(got, want) <= 1e-11


def test_spline_weights_reproduce_cubic_data():
    """Not-a-knot splines reproduce cubics exactly: the weights applied to
    samples of a cubic return the cubic at the query."""
    n, h = 9, 0.7
    xs = np.arange(n) * h
    f = lambda x: 0.3 - 1.1 * x + 0.25 * x * x - 0.05 * x ** 3
    for q in (0.0, 0.33, 2.9, 5.55, (n - 1) * h):
        w = O.spline_weights(n, 0.0, h, q)
        assert abs(float(w @ f(xs)) - f(q)) < 1e-12

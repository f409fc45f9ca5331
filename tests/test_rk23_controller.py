"""The adaptive RK23 step-size controller of the device integrator
(wave-vortex-model_gb300/csrc/wv_rk23_controller.hpp), compiled with g++ and
driven by a host backend on the reference's known-answer systems
(PortableRuntime/tests/TestWVUnifiedIntegration.cpp:366-478)."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def kat(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("rk23") / "kat")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT}/include",
                           f"-I{ROOT}/wave-vortex-model_gb300/csrc", os.path.join(ROOT, "tests", "rk23_controller_kat.cpp"),
                           "-o", exe])
    out = subprocess.check_output([exe], text=True)
    return {r["case"]: r for r in map(json.loads, out.strip().splitlines())}


def test_matlab_ode23_parity(kat):
    """TestWVUnifiedIntegration.cpp:437-478: 159 accepted, 6 rejected, 496
    evaluations, first step 2^-7, endpoint of MATLAB's ode23 to 1e-14."""
    r = kat["ode23_parity"]
    assert r["rc"] == 0 and r["t"] == 1.0
    assert (r["accepted"], r["rejected"], r["evaluations"], r["diagnostics"]) == (159, 6, 496, 159)
    assert abs(r["first_step"] - 0.0078125) < 1e-15
    assert abs(r["y0"][0] - 0.36787943731476008) < 1e-14
    assert abs(r["y0"][1] - 0.18393971865738004) < 1e-14


def test_zero_derivative_work(kat):
    """TestWVUnifiedIntegration.cpp:402-435: maximum step 0.1 over [0, 1]: 10
    accepted, no rejection, 31 evaluations (first same as last), zero error."""
    r = kat["zero_derivative"]
    assert r["rc"] == 0
    assert (r["accepted"], r["rejected"], r["evaluations"], r["diagnostics"]) == (10, 0, 31, 10)
    assert abs(r["first_step"] - 0.1) < 1e-14
    assert r["max_diag_error"] == 0.0
    assert r["first_fsal"] == 0 and r["last_fsal"] == 1


def test_rejection_without_growth_and_dense_output(kat):
    """TestWVUnifiedIntegration.cpp:366-390: a rejected first attempt, no step
    growth right after a rejection, dense output at the midpoint within 1e-6
    of exp(-t)."""
    r = kat["single_step"]
    assert r["rc"] == 0
    assert r["rejected"] > 0 and r["accepted"] == 1
    assert abs(r["next"] - r["last_step"]) < 1e-15
    assert abs(r["dense0"]) < 1e-6

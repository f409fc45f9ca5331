"""Adaptive RK23 on the GPU (wv_rk23_*, through the C ABI) against runs of the
reference integrator WVAdaptiveRK23 on the wave-vortex system
(tests/golden/rk23.npz, PortableRuntime/src/WVRungeKutta.cpp:554-983): the same
accepted/rejected/evaluation counts, tolerance audit hashes bit for bit, step
sizes to FP64 noise, end state and dense output at the FP64 parity gate."""
import math

import numpy as np
import pytest

from _cases import FP64_REL_TOL, RK23_RUNS, config_from_case, rel_err, rk23_run, state_components_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def _kernel(wv, cf, precision="fp64"):
    c = config_from_case(cf)
    k = wv.WVTransformConstantStratificationKernel(
        wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                         planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                         isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias), precision=precision)
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    return k


def _options(wv, o):
    return wv.WVAdaptiveRK23Options(relativeTolerance=o["rtol"], absoluteToleranceScale=o["atol_scale"],
                                    safetyFactor=o["safety"], rejectionFloorFactor=o["floor"],
                                    maximumStepFactor=o["max_factor"], maximumStepSize=o["max_step"])


@pytest.mark.parametrize("key", sorted(RK23_RUNS))
def test_rk23_matches_reference_integrator(wv, key):
    import torch
    cf, o, ref = rk23_run(key)
    k = _kernel(wv, cf)
    rk = wv.WVAdaptiveRK23(k, _options(wv, o))
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    t = rk.advanceToTime(*y, ref["t"], ref["t0"], ref["final"], ref["initial"])
    torch.cuda.synchronize()
    assert t == ref["tout"]
    m = rk.metrics()
    assert [m["accepted_steps"], m["rejected_steps"], m["rhs_evaluations"], m["fsal_reuses"]] == ref["counts"].tolist()
    h, per = rk.toleranceHash()
    assert [h] + per == [int(v) for v in ref["hashes"]]
    diag = rk.stepDiagnostics()
    assert len(diag) == len(ref["diag"])
    for d, r in zip(diag, ref["diag"]):
        assert d["rejectedAttemptCount"] == r[4] and d["rightHandSideEvaluationCount"] == r[5]
        assert d["reusedFSALDerivative"] == bool(r[6])
        assert abs(d["acceptedStepSize"] - r[1]) <= 1e-6 * r[1]
        assert abs(d["initialTime"] - r[0]) <= 1e-6 * max(1.0, abs(r[0]))
    assert abs(rk.nextStepSize() - ref["next"]) <= 1e-6 * ref["next"]
    assert not state_components_close([x.cpu().numpy() for x in y], ref, ("Kp", "Km", "K0"), 1e-11)
    dense = rk.evaluateDenseOutput(ref["dense_time"])
    want = {str(i): np.asarray(ref["dense"][i]) for i in range(3)}
    assert not state_components_close([x.cpu().numpy() for x in dense], want, ("0", "1", "2"), 1e-11)
    assert rk.metrics()["dense_output_evaluations"] == 1
    rk.close()
    k.close()


def test_host_entry_matches_device_entry(wv):
    import torch
    cf, o, ref = rk23_run("odd")
    k = _kernel(wv, cf)
    a = wv.WVAdaptiveRK23(k, _options(wv, o))
    Ap, Am, A0, t = a.advanceToTime(ref["Ap"], ref["Am"], ref["A0"], ref["t"], ref["t0"], ref["final"], ref["initial"])
    b = wv.WVAdaptiveRK23(k, _options(wv, o))
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    b.advanceToTime(*y, ref["t"], ref["t0"], ref["final"], ref["initial"])
    torch.cuda.synchronize()
    for host, dev in zip((Ap, Am, A0), y):
        assert np.array_equal(host, dev.cpu().numpy())
    assert a.metrics()["rhs_evaluations"] == b.metrics()["rhs_evaluations"]
    a.close()
    b.close()
    k.close()


def test_single_steps_follow_the_controller(wv):
    """step() repeated with nextStepSize() reproduces advanceToTime's first steps
    (first same as last from the second step on)."""
    import torch
    cf, o, ref = rk23_run("odd")
    k = _kernel(wv, cf)
    rk = wv.WVAdaptiveRK23(k, _options(wv, o))
    assert rk.lastAcceptedStep() is None
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    t, h = ref["t"], ref["initial"]
    for i in range(4):
        t_new = rk.step(*y, t, ref["t0"], h)
        assert rk.lastAcceptedStep() == (t, t_new)
        assert abs((t_new - t) - ref["diag"][i, 1]) <= 1e-6 * ref["diag"][i, 1]
        t, h = t_new, rk.nextStepSize()
    diag = rk.stepDiagnostics()
    assert [d["reusedFSALDerivative"] for d in diag] == [False, True, True, True]
    rk.prepareStateAfterRestart()
    assert rk.lastAcceptedStep() is None and rk.stepDiagnostics() == []
    rk.close()
    k.close()


def test_errors(wv):
    import torch
    cf, o, ref = rk23_run("odd")
    k = _kernel(wv, cf)
    with pytest.raises(wv.WVKernelError) as e:
        wv.WVAdaptiveRK23(k, wv.WVAdaptiveRK23Options(safetyFactor=1.5))
    assert e.value.code == 1
    rk = wv.WVAdaptiveRK23(k)
    with pytest.raises(wv.WVKernelError) as e:
        rk.evaluateDenseOutput(0.0)
    assert e.value.code == 10
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    with pytest.raises(wv.WVKernelError) as e:
        rk.advanceToTime(*y, 10.0, 0.0, 5.0, 1.0)
    assert e.value.code == 1
    with pytest.raises(wv.WVKernelError) as e:
        rk.step(*y, 0.0, 0.0, math.nan)
    assert e.value.code == 1
    t = rk.step(*y, 0.0, 0.0, 5.0)
    with pytest.raises(wv.WVKernelError) as e:
        rk.evaluateDenseOutput(t + 1.0)
    assert e.value.code == 1
    rk.close()
    k.close()


def test_mixed_precision_rk23_tracks_fp64(wv):
    """A mixed-precision handle under the same controller: the change of the
    state over the run agrees with the FP64 reference run to within the mixed
    form's flux accuracy (1e-2 of the change, the w and eta tendencies being
    the least accurate at about 1e-3)."""
    import torch
    cf, o, ref = rk23_run("odd")
    k = _kernel(wv, cf, precision="mixed")
    rk = wv.WVAdaptiveRK23(k, _options(wv, o))
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    rk.advanceToTime(*y, ref["t"], ref["t0"], ref["final"], ref["initial"])
    torch.cuda.synchronize()
    m = rk.metrics()
    assert abs(int(m["accepted_steps"]) - int(ref["counts"][0])) <= 2
    for got, want, init in zip(y, (ref["Kp"], ref["Km"], ref["K0"]), (ref["Ap"], ref["Am"], ref["A0"])):
        err = np.linalg.norm(got.cpu().numpy() - want) / np.linalg.norm(want - init)
        print("mixed RK23 end state error relative to the state change:", err)
        assert err <= 1e-2
    rk.close()
    k.close()


@pytest.mark.parametrize("key", ["odd", "hd"])
def test_rk4_advance_to_time_and_dense_output(wv, key):
    """WVFixedStepRK4::advanceToTime with a final partial step and the retained
    dense output, against the reference integrator (tests/golden/rk4_dense.npz)."""
    import torch
    from _cases import rk4_dense_run
    cf, g = rk4_dense_run(key)
    k = _kernel(wv, cf)
    k.set_forcing(nonlinear=True, adaptive_damping=bool(g["damping"]))
    with pytest.raises(wv.WVKernelError) as e:
        k.rk4DenseOutput(float(g["dense_time"]))
    assert e.value.code == 10
    k.setRK4DenseOutput(True)
    y = [torch.from_numpy(np.ascontiguousarray(g[n])).cuda() for n in ("Ap", "Am", "A0")]
    t = k.rk4AdvanceToTime(*y, float(g["t"]), float(g["t0"]), float(g["final"]), float(g["dt"]))
    assert t == float(g["tout"])
    assert not state_components_close([x.cpu().numpy() for x in y], g, ("Kp", "Km", "K0"), FP64_REL_TOL)
    dense = k.rk4DenseOutput(float(g["dense_time"]))
    for got, want in zip(dense, g["dense"]):
        assert rel_err(got.cpu().numpy(), want) <= FP64_REL_TOL
    with pytest.raises(wv.WVKernelError) as e:
        k.rk4DenseOutput(float(g["final"]) + 1.0)
    assert e.value.code == 1
    # host-pointer form: the same result
    Hp, Hm, H0, th = k.rk4AdvanceToTime(g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]), float(g["final"]),
                                        float(g["dt"]))
    assert th == t
    for a, b in zip((Hp, Hm, H0), y):
        assert np.array_equal(a, b.cpu().numpy())
    k.close()

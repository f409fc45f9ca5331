"""Integration systems with integrated observers on the GPU (wv_system_*,
through the C ABI) against the reference's WVConstantStratificationIntegrationSystem
(tests/golden/system.npz): the right-hand side (flux, particle velocities with
linear and spline sampling, F-grid tracer advection from the shared advection
fields), RK4 steps and an adaptive RK23 interval over the packed state."""
import numpy as np
import pytest

from _cases import config_from_case, rel_err, system_run

pytestmark = pytest.mark.gpu

RUNS = ["obs", "hd"]


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def _system(wv, key):
    cf, run, g = system_run(key)
    c = config_from_case(cf)
    k = wv.WVTransformConstantStratificationKernel(
        wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                         planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                         isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias))
    k.set_forcing(nonlinear=True, adaptive_damping=run["schedule"] == 1)
    groups = [wv.WVParticleGroup(x=gr["x"], y=gr["y"], z=gr["z"], isXYOnly=gr["xy_only"],
                                 advectionInterpolation="spline" if gr["spline"] else "linear",
                                 horizontalAbsoluteTolerance=gr["tol_h"], verticalAbsoluteTolerance=gr["tol_v"])
              for gr in run["groups"]]
    tracers = [wv.WVTracerSpec(shouldAntialias=t["antialias"], absoluteTolerance=t["tol"]) for t in run["tracers"]]
    s = wv.WVConstantStratificationIntegrationSystem(k, groups, tracers)
    return k, s, run, g


def _compare(s, got, want, coeff_tol, block_tol):
    M2 = 2 * int(np.prod(s.kernel.spectral_shape))
    for i in range(3):
        assert rel_err(got[i * M2:(i + 1) * M2], want[i * M2:(i + 1) * M2]) <= coeff_tol, i
    for o, n in zip(s.block_offsets, s.block_lengths):
        assert rel_err(got[o:o + n], want[o:o + n]) <= block_tol, (o, n, rel_err(got[o:o + n], want[o:o + n]))


@pytest.mark.parametrize("key", RUNS)
def test_system_rhs_matches_reference(wv, key):
    import torch
    k, s, run, g = _system(wv, key)
    state = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Ap", "Am", "A0")] + [g["extra"]])
    assert state.size == s.state_doubles
    x = torch.from_numpy(state).cuda()
    r = s.evaluateRightHandSide(float(g["t"]), float(g["t0"]), x).cpu().numpy()
    want = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Fp", "Fm", "F0")] + [g["rhs_extra"]])
    _compare(s, r, want, 1e-12, 1e-11)
    # the accepted state is not modified (particle positions stay unwrapped)
    assert np.array_equal(x.cpu().numpy(), state)
    s.close()
    k.close()


@pytest.mark.parametrize("key", RUNS)
def test_system_rk4_matches_reference(wv, key):
    import torch
    k, s, run, g = _system(wv, key)
    state = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Ap", "Am", "A0")] + [g["extra"]])
    x = torch.from_numpy(state).cuda()
    t = s.rk4(x, float(g["t"]), float(g["t0"]), float(g["dt"]), int(g["steps"]))
    assert t == float(g["k_t"])
    want = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Kp", "Km", "K0")] + [g["k_extra"]])
    got = x.cpu().numpy()
    _compare(s, got, want, 1e-12, 1e-12)
    # host-pointer entry: the same arithmetic
    host, th = s.rk4(state, float(g["t"]), float(g["t0"]), float(g["dt"]), int(g["steps"]))
    assert th == t and np.array_equal(host, got)
    s.close()
    k.close()


@pytest.mark.parametrize("key", RUNS)
def test_system_rk23_matches_reference(wv, key):
    import torch
    k, s, run, g = _system(wv, key)
    o = g["rk23_opts"]
    rk = wv.WVAdaptiveRK23(s, wv.WVAdaptiveRK23Options(relativeTolerance=float(o[0]), absoluteToleranceScale=float(o[1]),
                                                      safetyFactor=float(o[2]), rejectionFloorFactor=float(o[3]),
                                                      maximumStepFactor=float(o[4]), maximumStepSize=float(o[5])))
    state = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Ap", "Am", "A0")] + [g["extra"]])
    x = torch.from_numpy(state).cuda()
    t = rk.advanceToTime(x, float(g["t"]), float(g["t0"]), float(g["rk23_final"]), float(g["rk23_initial"]))
    torch.cuda.synchronize()
    assert t == float(g["r_t"])
    m = rk.metrics()
    assert [m["accepted_steps"], m["rejected_steps"], m["rhs_evaluations"], m["fsal_reuses"]] == g["r_counts"].tolist()
    steps = np.array([d["acceptedStepSize"] for d in rk.stepDiagnostics()])
    assert np.max(np.abs(steps - g["r_steps"]) / g["r_steps"]) < 1e-6
    want = np.concatenate([np.ascontiguousarray(g[n]).view(np.float64).ravel() for n in ("Rp", "Rm", "R0")] + [g["r_extra"]])
    _compare(s, x.cpu().numpy(), want, 1e-11, 1e-11)
    # dense output at the end of the last step is the accepted state
    ti, tf = rk.lastAcceptedStep()
    assert np.allclose(rk.evaluateDenseOutput(tf).cpu().numpy(), x.cpu().numpy(), rtol=0, atol=1e-14 * np.abs(want).max())
    rk.close()
    s.close()
    k.close()


def test_system_rejects_wrong_state(wv):
    import torch
    k, s, run, g = _system(wv, "obs")
    with pytest.raises(wv.WVKernelError) as e:
        s.evaluateRightHandSide(0.0, 0.0, torch.zeros(s.state_doubles + 1, dtype=torch.float64, device="cuda"))
    assert e.value.code == 2
    rk = wv.WVAdaptiveRK23(k)
    with pytest.raises(wv.WVKernelError):
        rk._lib.wv_rk23_system_step_device  # the coefficient integrator has no packed-state form
        x = torch.zeros(s.state_doubles, dtype=torch.float64, device="cuda")
        import ctypes
        tt = ctypes.c_double(0.0)
        rk._check(rk._lib.wv_rk23_system_step_device(rk._h, x.data_ptr(), ctypes.byref(tt), 0.0, 1.0, None))
    rk.close()
    s.close()
    k.close()

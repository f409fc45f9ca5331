"""Fixed-step RK4 contract on the GPU (UnitTests/TestWVModelIntegration.m:18-48,
PortableRuntime/tests/TestWVForcingAndRK4.cpp:276-305).

  * Segmented integration (to the checkpoint time, then on to the final time)
    equals uninterrupted integration bit for bit, and so does a restart from the
    checkpoint state in a new handle (the reference's checkpoint is a NetCDF
    file; here the caller's arrays carry the state).
  * Fixed steps converge at fourth order: errors of dt = 20 s and dt = 10 s
    against a tight reference have a ratio in [8, 24] and the fine error is at
    most 2e-8 of the largest coefficient (the reference's bounds).  The tight
    reference is the same integrator at dt = 1.25 s (the reference uses its
    adaptive integrator at atol 1e-12 / rtol 1e-10; either sits far below the
    fine error).

Workload: 16x16x9 and 32x32x17 over 40 km x 40 km x 1 km, N0 5.2e-3, latitude
45 (the single-wave 16x16x9 domain), seeded spectrum state at 1 m/s rms (strong enough
that truncation error sits far above paired-FP32 rounding), t = 0 .. 600 s,
checkpoint at 300 s; schedule {nonlinear advection, adaptive damping} for the
segmented / restarted runs, nonlinear advection for the convergence order.
"""
import numpy as np
import pytest

import wv_oracle as O

pytestmark = pytest.mark.gpu

FINAL, CHECKPOINT = 600.0, 300.0
GRIDS = [(16, 9), (32, 17)]


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def _setup(wv, N, Nz, precision, damping=True):
    c = O.Config(Nx=N, Ny=N, Nz=Nz, Nj=O.default_nj(Nz), Lx=40e3, Ly=40e3, Lz=1000.0, N0=5.2e-3, latitude=45.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=7, urms=1.0)
    k = wv.WVTransformConstantStratificationKernel(wv.Configuration(
        Nx=N, Ny=N, Nz=Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, latitude=c.latitude), precision=precision)
    k.set_forcing(nonlinear=True, adaptive_damping=damping)
    return c, d, A, k


def _run(k, A, t, dt, until):
    steps = int(round((until - t) / dt))
    Ap, Am, A0, t = k.rk4(*A, t, 0.0, dt, steps)
    return (Ap, Am, A0), t


@pytest.mark.parametrize("precision", ["fp64", "fp32x2", "mixed"])
@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: f"{g[0]}x{g[0]}x{g[1]}")
def test_segmented_and_restarted_equal_uninterrupted(wv, grid, precision):
    c, d, A, k = _setup(wv, *grid, precision)
    dt = 10.0
    whole, tw = _run(k, A, 0.0, dt, FINAL)
    half, th = _run(k, A, 0.0, dt, CHECKPOINT)
    assert th == CHECKPOINT
    seg, ts = _run(k, half, th, dt, FINAL)
    assert tw == ts == FINAL
    for a, b in zip(seg, whole):
        assert np.array_equal(a, b)
    # restart: the checkpoint state copied out and integrated by a new handle
    _, _, _, k2 = _setup(wv, *grid, precision)
    restarted, tr = _run(k2, [np.array(x, copy=True) for x in half], CHECKPOINT, dt, FINAL)
    assert tr == FINAL
    for a, b in zip(restarted, whole):
        assert np.array_equal(a, b)
    # invariants: finite, waves present, no wave amplitude at j = 0 for Kh > 0
    assert all(np.all(np.isfinite(x)) for x in whole)
    assert np.max(np.abs(whole[0])) > 0 and np.max(np.abs(whole[1])) > 0
    wavesAtJ0 = d.Kh > 0
    assert not np.any(whole[0][wavesAtJ0, 0]) and not np.any(whole[1][wavesAtJ0, 0])
    k.close()
    k2.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32x2"])
@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: f"{g[0]}x{g[0]}x{g[1]}")
def test_fixed_step_converges_at_fourth_order(wv, grid, precision):
    # nonlinear advection alone: adaptive damping scales the flux by max |u_h|
    # over the grid, which is only piecewise smooth in the state (its arg max
    # can move between stages), so with it the observed order falls below four
    c, d, A, k = _setup(wv, *grid, precision, damping=False)

    def err(a, b):
        return max(np.max(np.abs(x - y)) for x, y in zip(a, b)) / max(max(np.max(np.abs(y)) for y in b),
                                                                       np.finfo(float).eps)

    ref, _ = _run(k, A, 0.0, 1.25, FINAL)
    coarse, _ = _run(k, A, 0.0, 20.0, FINAL)
    fine, _ = _run(k, A, 0.0, 10.0, FINAL)
    ec, ef = err(coarse, ref), err(fine, ref)
    assert ef <= 2e-8, ef
    assert 8.0 <= ec / ef <= 24.0, (ec, ef, ec / ef)
    k.close()

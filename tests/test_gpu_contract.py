"""Failure-path contract of the C ABI, through the library's test hooks (host-side
failure injection; no GPU fault, no hang).

Reference contract tests followed:
  * an injected allocation failure during kernel creation is reported as
    allocationFailure, yields no kernel and leaks nothing
    (tools/compiled-kernel/tests/TestWVKernelContract.cpp:331-340);
  * an injected execution failure is reported as fftExecutionFailure and the
    kernel stays usable (TestWVKernelContract.cpp:342-355);
  * a failed RK4 step leaves the caller's state and time untouched
    (PortableRuntime/tests/TestWVForcingAndRK4.cpp:307-319);
  * operations on one kernel are not reentrant (ExecutionGuard,
    CompiledKernel/src/WVTransformConstantStratificationKernel.cpp:76-84).
Plus the GPU side of failure detection: the tensor-core vertical inverse's
bounded mbarrier wait is made to run out before any MMA is issued; the kernel
records it in the device status word, frees its tensor memory and returns, and
the handle stays usable.
"""
import ctypes
import gc

import numpy as np
import pytest

import wv_oracle as O
from _cases import rel_err

pytestmark = pytest.mark.gpu

WV_ALLOCATION_FAILURE = 6
WV_FFT_EXECUTION_FAILURE = 8
WV_REENTRANT_EXECUTION = 11


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def _config(wv, N=48, Nz=25):
    return wv.Configuration(Nx=N, Ny=N, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * N, Ly=3125.0 * N, Lz=4000.0,
                            latitude=33.0)


def _state(c, seed=3):
    d = O.build_descriptor(O.Config(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, latitude=c.latitude))
    return d, O.spectrum_state(d, seed=seed, urms=0.1)


@pytest.mark.parametrize("n", [0, 1, 7, 25])
def test_allocation_failure_on_create_leaks_nothing(wv, n):
    lib = wv.load_library()
    cfg = _config(wv)
    # handles of earlier tests are released now, not by a collection during this test
    gc.collect()
    gc.disable()
    try:
        baseline = lib.wv_test_live_device_bytes()
        h = ctypes.c_void_p()
        lib.wv_test_fail_allocation_after(n)
        try:
            rc = lib.wv_create(ctypes.byref(cfg._c()), 0, ctypes.byref(h))
        finally:
            lib.wv_test_fail_allocation_after(-1)
        assert rc == WV_ALLOCATION_FAILURE
        assert not h.value
        assert lib.wv_test_live_device_bytes() == baseline
        # the library is still usable, and a created handle's bytes are returned on destroy
        k = wv.WVTransformConstantStratificationKernel(cfg)
        assert lib.wv_test_live_device_bytes() == baseline + k.metrics()["device_bytes"]
        k.close()
        assert lib.wv_test_live_device_bytes() == baseline
    finally:
        gc.enable()


def test_injected_execution_failure_is_reported_and_handle_stays_usable(wv):
    c = _config(wv)
    d, A = _state(c)
    k = wv.WVTransformConstantStratificationKernel(c)
    expected = k.nonlinearFlux(0.0, 0.0, *A)
    k._lib.wv_test_fail_launch_after(k._h, 0)
    with pytest.raises(wv.WVKernelError) as err:
        k.nonlinearFlux(0.0, 0.0, *A)
    assert err.value.code == WV_FFT_EXECUTION_FAILURE
    assert "injected execution failure" in str(err.value)
    assert err.value.identifier == "WaveVortexModel:CompiledKernelExecution"
    # one-shot: the next call runs and gives the same flux
    for a, b in zip(k.nonlinearFlux(0.0, 0.0, *A), expected):
        assert np.array_equal(a, b)
    k.close()


@pytest.mark.parametrize("entry", ["host", "device"])
def test_failed_rk4_leaves_caller_state_and_time_untouched(wv, entry):
    import torch
    c = _config(wv)
    d, A = _state(c)
    dt = O.cfl_time_step(d, *A)
    k = wv.WVTransformConstantStratificationKernel(c)
    lib = k._lib
    before = [np.ascontiguousarray(a).copy() for a in A]
    t = ctypes.c_double(250.0)
    # the first step's first two right-hand sides run, the third fails
    lib.wv_test_fail_launch_after(k._h, 2)
    if entry == "host":
        arrays = [np.ascontiguousarray(a).copy() for a in A]
        rc = lib.wv_rk4_steps(k._h, *(a.ctypes.data for a in arrays), ctypes.byref(t), ctypes.c_double(0.0),
                              ctypes.c_double(dt), 2)
        after = arrays
    else:
        dev = [torch.from_numpy(a.copy()).cuda() for a in before]
        rc = lib.wv_rk4_steps_device(k._h, *(x.data_ptr() for x in dev), ctypes.byref(t), ctypes.c_double(0.0),
                                     ctypes.c_double(dt), 2, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        after = [x.cpu().numpy() for x in dev]
    assert rc == WV_FFT_EXECUTION_FAILURE
    assert "injected execution failure" in lib.wv_last_message(k._h).decode()
    assert t.value == 250.0
    for a, b in zip(after, before):
        assert np.array_equal(a, b)
    # the handle steps normally afterwards, exactly as a fresh handle does
    Kp, Km, K0, t1 = k.rk4(*before, 250.0, 0.0, dt, 1)
    k2 = wv.WVTransformConstantStratificationKernel(c)
    Rp, Rm, R0, t2 = k2.rk4(*before, 250.0, 0.0, dt, 1)
    assert t1 == t2
    for a, b in zip((Kp, Km, K0), (Rp, Rm, R0)):
        assert np.array_equal(a, b)
    k.close()
    k2.close()


def test_reentrant_call_is_rejected(wv):
    c = _config(wv)
    d, A = _state(c)
    k = wv.WVTransformConstantStratificationKernel(c)
    k._lib.wv_test_hold_busy(k._h, 1)
    try:
        for call in (lambda: k.nonlinearFlux(0.0, 0.0, *A), lambda: k.rk4(*A, 0.0, 0.0, 10.0, 1),
                     lambda: k.transformWaveVortexToUVWEta(0.0, 0.0, *A)):
            with pytest.raises(wv.WVKernelError) as err:
                call()
            assert err.value.code == WV_REENTRANT_EXECUTION
            assert "reentrant" in str(err.value)
    finally:
        k._lib.wv_test_hold_busy(k._h, 0)
    F = k.nonlinearFlux(0.0, 0.0, *A)
    G = O.nonlinear_flux(d, *A, 0.0, 0.0)
    for a, b in zip(F, G):
        assert rel_err(a, b) <= 1e-11
    k.close()


def test_bounded_wait_runs_out_reports_and_recovers(wv):
    """64x64x33 mixed handle on the tensor-core vertical inverse (k_vinv_tc):
    its first matrix-operand wait is armed without a copy and bounded to 64
    polls, so it runs out in every CTA before any MMA; the status word reports
    it, no call hangs, and after the hook is cleared the same handle's flux
    equals a fresh handle's bit for bit."""
    import torch
    c = _config(wv, 64, 33)
    d, A = _state(c, seed=5)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    k = wv.WVTransformConstantStratificationKernel(c, precision="mixed")
    k.set_vertical_kernel("tensor")
    k._lib.wv_reset_device_status(k._h)
    k._lib.wv_test_inject_wait_timeout(k._h, 64)
    try:
        k.nonlinearFlux(0.0, 0.0, *dev)
        torch.cuda.synchronize()
        assert k.device_status() & 1
    finally:
        k._lib.wv_test_inject_wait_timeout(k._h, 0)
    k._lib.wv_reset_device_status(k._h)
    assert k.device_status() == 0
    F = [x.cpu().numpy() for x in k.nonlinearFlux(0.0, 0.0, *dev)]
    fresh = wv.WVTransformConstantStratificationKernel(c, precision="mixed")
    fresh.set_vertical_kernel("tensor")
    G = [x.cpu().numpy() for x in fresh.nonlinearFlux(0.0, 0.0, *dev)]
    for a, b in zip(F, G):
        assert np.array_equal(a, b)
    assert k.device_status() == 0 and fresh.device_status() == 0
    # and it is the mixed flux (FP32 arithmetic): near the FP64 oracle's
    R = O.nonlinear_flux(d, *A, 0.0, 0.0)
    for a, b in zip(F, R):
        assert rel_err(a, b) <= 1e-2
    k.close()
    fresh.close()

"""The allocation-free flux entry point (wv_nonlinear_flux_device_noalloc).

Some callers cannot call cudaMalloc where they need a flux: a host application
whose memory manager owns all device memory and forbids further driver
allocations, or a loop that cannot afford cudaMalloc's implicit device
synchronization.  For them the library keeps the flux scratch in one static
device array.  This test calls that entry point through the C ABI and checks it
against the regular device entry point of the same handle, on two calls in a
row with different states (the shared array keeps the previous call's
contents), for every precision and vertical-kernel choice, on two grids, and
that configurations too large for the array are rejected with a clear error.

Collected last (file name) so a stop-at-first-failure run has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import wv_oracle as O
from _cases import FP64_REL_TOL, rel_err

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


def _config(wv, Nx, Ny, Nz):
    return wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=400e3, Ly=400e3 * Ny / Nx, Lz=4000.0,
                            latitude=33.0)


# (precision, vertical kernel): each precision's default, and the other kernels
# the handle can be switched to (the entry point follows the handle's choice)
VARIANTS = [("fp64", None), ("fp64", "cuda"), ("fp32x2", None), ("fp32x2", "tensor"), ("mixed", None),
            ("mixed", "tensor"), ("mixed", "cuda")]
# 64x64x33, and a rectangular odd grid (radix-3 and radix-5 FFTs, Nz = 25)
GRIDS = [(64, 64, 33), (60, 45, 25)]


@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("precision,vertical", VARIANTS, ids=lambda v: str(v))
def test_noalloc_flux_matches_device_entry_on_two_calls(wv, precision, vertical, grid):
    import torch
    c = _config(wv, *grid)
    d = O.build_descriptor(O.Config(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, latitude=c.latitude))
    k = wv.WVTransformConstantStratificationKernel(c, precision=precision)
    if vertical is not None:
        k.set_vertical_kernel(vertical)
    lib = wv.load_library()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for seed, (t, t0) in ((11, (500.0, 0.0)), (12, (1234.5, 10.0))):
        state = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in O.spectrum_state(d, seed=seed, urms=0.1)]
        expected = k.nonlinearFlux(t, t0, *state)
        got = tuple(torch.full_like(state[0], float("nan")) for _ in range(3))
        rc = lib.wv_nonlinear_flux_device_noalloc(k._h, t, t0, *(s.data_ptr() for s in state),
                                                  *(g.data_ptr() for g in got), stream)
        assert rc == 0, lib.wv_last_message(k._h).decode()
        torch.cuda.synchronize()
        for a, b in zip(got, expected):
            a, b = a.cpu().numpy(), b.cpu().numpy()
            assert np.all(np.isfinite(a))
            # same kernels on the same inputs: within the FP64 gate (in practice bit for bit)
            assert rel_err(a, b) <= FP64_REL_TOL
    assert k.device_status() == 0
    k.close()


def test_noalloc_rejects_configurations_beyond_the_static_array(wv):
    import torch
    c = _config(wv, 256, 256, 129)
    k = wv.WVTransformConstantStratificationKernel(c)
    lib = wv.load_library()
    z = torch.zeros(k.spectral_shape, dtype=torch.complex128, device="cuda")
    out = [torch.empty_like(z) for _ in range(3)]
    rc = lib.wv_nonlinear_flux_device_noalloc(k._h, 0.0, 0.0, z.data_ptr(), z.data_ptr(), z.data_ptr(),
                                              *(o.data_ptr() for o in out),
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 5  # WV_SIZE_OVERFLOW
    assert "static scratch array holds" in lib.wv_last_message(k._h).decode()
    k.close()

"""Several live handles of different grid sizes in one process.  Kernel
attributes such as the dynamic shared-memory cap belong to the kernel, not to a
handle: a handle created later for a smaller grid must leave a larger live
handle's launches valid (same results, bit for bit)."""
import numpy as np
import pytest

import wv_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available()
    build.build()
    return wvgpu


def _cfg(wv, Nx, Nz):
    return wv.Configuration(Nx=Nx, Ny=Nx, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Nx, Lz=4000.0,
                            latitude=33.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_small_handle_after_large_one(wv, precision):
    import torch
    big = wv.WVTransformConstantStratificationKernel(_cfg(wv, 256, 129), precision=precision)
    A = wv.synthetic_state(big, seed=5, urms=0.1)
    dA = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    first = [x.cpu().numpy() for x in big.nonlinearFlux(100.0, 0.0, *dA)]
    small = wv.WVTransformConstantStratificationKernel(_cfg(wv, 32, 17), precision=precision)
    As = wv.synthetic_state(small, seed=6, urms=0.1)
    small.nonlinearFlux(0.0, 0.0, *As)
    # adjoint kernels as well: the small handle's adjoint set-up comes first
    cs = small.flux_vjp(0.0, 0.0, *(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in As),
                        *(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in As))
    torch.cuda.synchronize()
    again = [x.cpu().numpy() for x in big.nonlinearFlux(100.0, 0.0, *dA)]
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    cb = big.flux_vjp(100.0, 0.0, *dA, *dA)
    torch.cuda.synchronize()
    assert all(np.isfinite(x.cpu().numpy()).all() for x in cb + cs)
    # the host-pointer RK4 path of the larger handle after the smaller one
    Ap, Am, A0, t = big.rk4(*A, 0.0, 0.0, 60.0, 1)
    assert t == 60.0 and np.isfinite(Ap).all()
    small.close()
    big.close()

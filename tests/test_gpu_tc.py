"""Tensor-core vertical transforms (tcgen05.mma, split-BF16 with FP32
accumulators; the inverse k_vinv_tc and the forward k_vfwd_tc)
of the mixed-form flux against the CUDA-core kernels.  Both are
FP32 computations that differ in rounding order; each is measured against the
FP64 flux as field tendencies (u, v, w, eta through the FP64 inverse transform)
and the tensor-core error must stay within a small factor of the CUDA-core
error.  The device status word (bounded waits) must stay clear."""
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


def _cfg(wv, Nx, Ny, Nz, hydro=False):
    return wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0,
                            latitude=33.0, isHydrostatic=hydro)


@pytest.mark.parametrize("Nx,Ny,Nz,hydro", [(32, 32, 17, False), (48, 40, 25, False), (64, 64, 33, False),
                                            (48, 40, 24, False), (64, 64, 64, True), (128, 128, 65, True),
                                            (96, 96, 97, False), (256, 256, 129, False)])
def test_tensor_core_vertical_matches_cuda_cores(wv, Nx, Ny, Nz, hydro):
    import torch
    cfg = _cfg(wv, Nx, Ny, Nz, hydro)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="mixed")
    A = wv.synthetic_state(k64, seed=21, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    exact = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in k64.nonlinearFlux(777.0, 5.0, *dev)))
    nf = 3 if hydro else 4
    fields = [0, 1, 3] if hydro else [0, 1, 2, 3]

    def tendency_error(F):
        f = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in F))
        return [float(np.linalg.norm(f[i] - exact[i]) / np.linalg.norm(exact[i])) for i in fields]

    k.set_vertical_kernel("cuda")
    ref = [x.clone() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    e_cuda = tendency_error(ref)
    k.set_vertical_kernel("tensor")
    e_tc = tendency_error(k.nonlinearFlux(777.0, 5.0, *dev))
    assert k.device_status() == 0
    print(f"{Nx}x{Ny}x{Nz} hydro={hydro} flux tendency error vs FP64 (u, v, [w,] eta): CUDA cores {e_cuda}, tensor cores {e_tc}")
    assert len(e_tc) == nf
    for a, b in zip(e_tc, e_cuda):
        assert a <= 3.0 * b + 1e-7
    # the switch back restores the CUDA-core path bit for bit
    k.set_vertical_kernel("cuda")
    again = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    for a, b in zip(again, ref):
        assert np.array_equal(a, b.cpu().numpy())
    k.close()
    k64.close()


def test_tensor_core_flux_error_vs_oracle(wv):
    """Field tendencies of the tensor-core mixed flux against the FP64 oracle: the
    same bounds as the CUDA-core mixed form."""
    c = O.Config(Nx=64, Ny=64, Nz=33, Nj=21, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=7, urms=0.1)
    k = wv.WVTransformConstantStratificationKernel(
        wv.Configuration(Nx=64, Ny=64, Nz=33, Nj=21, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0), precision="mixed")
    k.set_vertical_kernel("tensor")
    F = k.nonlinearFlux(1234.5, 10.0, *A)
    R = O.nonlinear_flux(d, *A, 1234.5, 10.0)
    fF = O.inverse_uvweta(d, *F, 0.0, 0.0)
    fR = O.inverse_uvweta(d, *R, 0.0, 0.0)
    err = [float(np.linalg.norm(fF[i] - fR[i]) / np.linalg.norm(fR[i])) for i in range(4)]
    print("tensor-core mixed flux tendency relative L2 error (u, v, w, eta):", err)
    assert max(err[0], err[1]) <= 2e-6
    assert max(err[2], err[3]) <= 1e-3
    assert k.device_status() == 0
    k.close()


def test_tensor_core_option_rejected_on_fp64(wv):
    k = wv.WVTransformConstantStratificationKernel(_cfg(wv, 32, 32, 17), precision="fp64")
    with pytest.raises(wv.WVKernelError) as e:
        k.set_vertical_kernel("tensor")
    assert e.value.code == 10
    k.close()


def test_tensor_core_members(wv):
    """Member-batched handles (ensemble groups) on the tensor-core kernel step every
    member exactly as a single-state handle on the tensor-core kernel does."""
    import torch
    cfgs = [_cfg(wv, 64, 64, 33), _cfg(wv, 48, 40, 25)]
    ens = wv.WVEnsemble(cfgs, [3, 2], precision="mixed", autotune=False)
    ens.set_vertical_kernel("tensor")
    X, singles = [], []
    for g, cfg in enumerate(cfgs):
        k = wv.WVTransformConstantStratificationKernel(cfg, precision="mixed")
        k.set_vertical_kernel("tensor")
        B = ens.members[g]
        X.append(torch.from_numpy(np.stack([np.stack(wv.synthetic_state(k, seed=40 + 7 * g + m, urms=0.1))
                                            for m in range(B)])).cuda())
        singles.append(k)
    Xe = [x.clone() for x in X]
    ens.rk4(Xe, 0.0, 0.0, [300.0, 250.0], 2)
    torch.cuda.synchronize()
    for g, (k, x0, xe) in enumerate(zip(singles, X, Xe)):
        for m in range(x0.shape[0]):
            s = [x0[m, c].clone() for c in range(3)]
            k.rk4(*s, 0.0, 0.0, [300.0, 250.0][g], 2)
            torch.cuda.synchronize()
            for c in range(3):
                assert torch.equal(s[c], xe[m, c]), (g, m, c)
        assert k.device_status() == 0
        k.close()
    assert [t["vertical"] for t in ens.tuning()] == ["tensor", "tensor"]
    ens.close()

"""Vertical transforms of the flux as FFTs of the even / odd extension over z
(WV_VERTICAL_FFT: the shared-memory k_vinv_fft, k_vfwd_fft, and on mixed and
FP32X2 handles with 2 (Nz - 1) = 32 R the warp-register k_vinv_wfft,
k_vfwd_wfft and the VJP's k_vfwd_adj_wfft, k_vinv_adj_wfft): every
reference golden case at the FP64 (1e-12) and FP32X2 (1e-9) tolerances (RK4
components that are pure accumulated rounding gated against the state), and
the flux against the dense folded contraction of the same handle on 0.1 m/s
spectrum states (odd and even Nz, hydrostatic)."""
import numpy as np
import pytest

import wv_oracle as O
from _cases import config_from_case, golden_cases, load_golden, rel_err, state_components_close

pytestmark = pytest.mark.gpu

CASES = golden_cases()
TOL = {"fp64": 1e-12, "fp32x2": 1e-9}


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available()
    build.build()
    return wvgpu


def _conf(wv, c):
    return wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                            planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                            isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


@pytest.mark.parametrize("precision", ["fp64", "fp32x2"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_fft_vertical_matches_reference(wv, name, precision):
    cf = CASES[name]
    g = load_golden(name)
    tol = TOL[precision]
    k = wv.WVTransformConstantStratificationKernel(_conf(wv, config_from_case(cf)), precision=precision)
    k.set_vertical_kernel("fft")
    t, t0 = float(g["t"]), float(g["t0"])
    args = (t, t0, g["Ap"], g["Am"], g["A0"])
    for got, key in zip(k.nonlinearFlux(*args), ("Fp", "Fm", "F0")):
        assert rel_err(got, g[key]) <= tol, (name, key, rel_err(got, g[key]))
    Fw, adv = k.nonlinearFluxWithAdvectionFields(*args)
    for got, key in zip(Fw, ("with_Fp", "with_Fm", "with_F0")):
        assert rel_err(got, g[key]) <= tol, (name, key)
    assert rel_err(adv, g["with_fields"]) <= tol
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    for got, key in zip(k.evaluateRightHandSide(*args), ("Rp", "Rm", "R0")):
        assert rel_err(got, g[key]) <= tol, (name, key)
    Kp, Km, K0, tK = k.rk4(g["rk_Ap"], g["rk_Am"], g["rk_A0"], float(g["rk_t"]), float(g["rk_t0"]), float(g["rk_dt"]),
                           int(g["rk_steps"]))
    assert not state_components_close((Kp, Km, K0), g, ("Kp", "Km", "K0"), tol), name
    k.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32x2"])
@pytest.mark.parametrize("Nx,Ny,Nz,hydro", [(32, 32, 17, False), (48, 40, 24, False), (64, 64, 33, True),
                                            (64, 64, 64, False), (128, 128, 65, False)])
def test_fft_vertical_flux_matches_dense_contraction(wv, Nx, Ny, Nz, hydro, precision):
    """The flux with the FFT vertical transforms against the dense folded
    contraction of the same handle, on the oracle's 0.1 m/s spectrum state.
    The max-norm relative difference of two valid FP64 orderings of the flux is
    set by its ill-conditioned coefficients (high j, small K_h) and grows with
    the grid: the oracle measures it on the same state (its FFT against its
    dense vertical transforms, O.noise_floor: 1.1e-12 at 32x32x17, 1.3e-11 at
    64x64x64, 2e-11 at 128x128x65, 3e-10 at 256x256x129), and the GPU
    difference must stay within 3x that floor (FP64) or 300x (paired FP32,
    2^8 times FP64's unit roundoff)."""
    import torch
    c = O.Config(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0, latitude=33.0,
                 isHydrostatic=hydro)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=29, urms=0.1)
    _, floors = O.noise_floor(O.nonlinear_flux, d, *A, 777.0, 5.0)
    cfg = wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, latitude=33.0, isHydrostatic=hydro)
    k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    k.set_vertical_kernel("cuda")
    ref = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    k.set_vertical_kernel("fft")
    got = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    err = [rel_err(a, b) for a, b in zip(got, ref)]
    print(f"{precision} {Nx}x{Ny}x{Nz} hydro={hydro}: FFT vs dense flux difference {err}, oracle FP64 floor {floors}")
    factor = 3.0 if precision == "fp64" else 300.0
    for e, fl in zip(err, floors):
        assert e <= factor * fl + (1e-14 if precision == "fp64" else 1e-12)
    k.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32x2", 1e-9)])
def test_fft_vertical_tendencies_at_256(wv, precision, tol):
    """At 256x256x129 the flux's field tendencies (u, v, w, eta through the FP64
    inverse transform; well conditioned, unlike single coefficients) with the
    FFT vertical transforms against the dense contraction."""
    import torch
    cfg = wv.Configuration(Nx=256, Ny=256, Nz=129, Nj=O.default_nj(129), Lx=800e3, Ly=800e3, Lz=4000.0, latitude=33.0)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = k64 if precision == "fp64" else wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
    A = wv.synthetic_state(k64, seed=23, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]

    def tendencies(kind):
        k.set_vertical_kernel(kind)
        F = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
        return k64.transformWaveVortexToUVWEta(0.0, 0.0, *F)

    dense, fft = tendencies("cuda"), tendencies("fft")
    err = [float(np.linalg.norm(fft[i] - dense[i]) / np.linalg.norm(dense[i])) for i in range(4)]
    print(f"{precision} 256x256x129 FFT vs dense flux tendencies (u, v, w, eta): {err}")
    assert max(err) <= tol
    if k is not k64:
        k.close()
    k64.close()


def test_vertical_kernel_defaults(wv):
    """FP64 and FP32X2: FFTs in both directions wherever 3 <= Nz <= 513.
    Mixed: the inverse as FFTs from Nz = 97, dense below; the forward as FFTs
    from Nz = 65, dense below.  One setter for both directions, one for each,
    and the rejections."""
    cfg = wv.Configuration(Nx=32, Ny=32, Nz=17, Nj=10, Lx=100e3, Ly=100e3, Lz=4000.0, latitude=33.0)
    for precision, kinds in (("fp64", ("fft", "fft")), ("fp32x2", ("fft", "fft")), ("mixed", ("cuda", "cuda"))):
        k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
        assert k.vertical_kernels() == kinds, precision
        assert k.vertical_kernel() == kinds[0]
        k.close()
    for (n, nz), kinds in (((128, 65), ("cuda", "fft")), ((192, 97), ("fft", "fft")), ((256, 129), ("fft", "fft")),
                           ((64, 257), ("fft", "fft"))):
        c = wv.Configuration(Nx=n, Ny=n, Nz=nz, Nj=O.default_nj(nz), Lx=3125.0 * n, Ly=3125.0 * n, Lz=4000.0, latitude=33.0)
        k = wv.WVTransformConstantStratificationKernel(c, precision="mixed")
        assert k.vertical_kernels() == kinds, (n, nz)
        k.close()
    big = wv.Configuration(Nx=256, Ny=256, Nz=129, Nj=O.default_nj(129), Lx=800e3, Ly=800e3, Lz=4000.0, latitude=33.0)
    k = wv.WVTransformConstantStratificationKernel(big, precision="mixed")
    k.set_vertical_kernel("tensor")
    assert k.vertical_kernels() == ("tensor", "tensor")
    k.set_vertical_kernel("cuda")
    assert k.vertical_kernels() == ("cuda", "cuda")
    k.set_vertical_kernels("fft", "tensor")
    assert k.vertical_kernels() == ("fft", "tensor")
    k.close()
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    for inv, fwd in (("tensor", "fft"), ("fft", "tensor")):
        with pytest.raises(wv.WVKernelError) as e:
            k.set_vertical_kernels(inv, fwd)
        assert e.value.code == 10
    assert k.vertical_kernels() == ("fft", "fft")
    k.close()
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
    k.set_vertical_kernel("tensor")  # digit-sliced inverse; the forward transform keeps the dense contraction
    assert k.vertical_kernels() == ("tensor", "cuda")
    with pytest.raises(wv.WVKernelError):
        k.set_vertical_kernels("fft", "tensor")
    k.close()


@pytest.mark.parametrize("Nx,Ny,Nz,hydro", [(32, 32, 17, False), (48, 40, 24, False), (64, 64, 33, True),
                                            (128, 128, 65, False), (256, 256, 129, False), (128, 128, 257, False)])
def test_fft_vertical_mixed_matches_cuda_cores(wv, Nx, Ny, Nz, hydro):
    """Mixed handles (FP32 arithmetic): the flux's field tendencies (u, v, w,
    eta through the FP64 inverse transform) with the FFT vertical transforms
    against the FP64 flux, within a small factor of the dense CUDA-core
    contraction's error on the same handle; the switch back to the dense
    kernels restores their flux bit for bit.  Nz = 257 is past the tensor-core
    kernels' limit (Nz <= 255)."""
    import torch
    cfg = wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0,
                           latitude=33.0, isHydrostatic=hydro)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="mixed")
    A = wv.synthetic_state(k64, seed=21, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    exact = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in k64.nonlinearFlux(777.0, 5.0, *dev)))
    fields = [0, 1, 3] if hydro else [0, 1, 2, 3]

    def tendency_error(F):
        f = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in F))
        return [float(np.linalg.norm(f[i] - exact[i]) / np.linalg.norm(exact[i])) for i in fields]

    k.set_vertical_kernel("cuda")
    ref = [x.clone() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    e_cuda = tendency_error(ref)
    k.set_vertical_kernel("fft")
    assert k.vertical_kernel() == "fft"
    e_fft = tendency_error(k.nonlinearFlux(777.0, 5.0, *dev))
    print(f"mixed {Nx}x{Ny}x{Nz} hydro={hydro} flux tendency error vs FP64 (u, v, [w,] eta): "
          f"dense {e_cuda}, FFT {e_fft}")
    for a, b in zip(e_fft, e_cuda):
        assert a <= 3.0 * b + 1e-7
    k.set_vertical_kernel("cuda")
    again = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev)]
    for a, b in zip(again, ref):
        assert np.array_equal(a, b.cpu().numpy())
    k.close()
    k64.close()


def test_fft_vertical_mixed_vjp_matches_dense(wv):
    """Mixed handles: the flux VJP with the FFT vertical maps against the FP64
    VJP (same state and cotangent), within a small factor of the dense adjoint
    maps' error on the same handle."""
    import torch
    c = O.Config(Nx=64, Ny=64, Nz=33, Nj=O.default_nj(33), Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    rng = np.random.default_rng(9)
    A = O.spectrum_state(d, seed=3, urms=0.1)
    Fb = [rng.standard_normal((d.Nkl, c.Nj)) + 1j * rng.standard_normal((d.Nkl, c.Nj)) for _ in range(3)]
    ins = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (*A, *Fb)]
    cfg = wv.Configuration(Nx=64, Ny=64, Nz=33, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, latitude=33.0)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="mixed")
    exact = [x.cpu().numpy() for x in k64.flux_vjp(0.0, 0.0, *ins)]
    errs = {}
    for kind in ("cuda", "fft"):
        k.set_vertical_kernel(kind)
        got = [x.cpu().numpy() for x in k.flux_vjp(0.0, 0.0, *ins)]
        errs[kind] = [rel_err(g, e) for g, e in zip(got, exact)]
    print("mixed flux VJP vs FP64 (Apb, Amb, A0b): dense", errs["cuda"], "FFT", errs["fft"])
    # Each FFT line pairs a cosine-family channel with a sine-family one, so in
    # FP32 the smaller channel's rounding is relative to the larger one: the
    # FFT maps' Apb and Amb errors reach the level of the dense maps' A0b error
    # (both ~6e-5 here), within the mixed VJP's 1e-3 bound against FP64.
    assert max(errs["fft"]) <= 3.0 * max(errs["cuda"]) + 1e-6
    k.close()
    k64.close()

@pytest.mark.parametrize("inv,fwd", [("tensor", "fft"), ("fft", "tensor"), ("cuda", "fft"), ("fft", "cuda"), ("tensor", "cuda")])
def test_mixed_vertical_kernel_per_direction(wv, inv, fwd):
    """Mixed handles, each vertical direction on its own kernel
    (wv_set_vertical_kernels): the flux's field tendencies against the FP64 flux
    within a small factor of the dense contraction's error, the device status
    word clear (the tensor-core kernels' bounded waits), and the VJP following
    the chosen maps within the mixed VJP's bound."""
    import torch
    cfg = wv.Configuration(Nx=128, Ny=128, Nz=65, Nj=O.default_nj(65), Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="mixed")
    A = wv.synthetic_state(k64, seed=31, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    exact = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in k64.nonlinearFlux(777.0, 5.0, *dev)))

    def tendency_error():
        F = k.nonlinearFlux(777.0, 5.0, *dev)
        f = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in F))
        return [float(np.linalg.norm(f[i] - exact[i]) / np.linalg.norm(exact[i])) for i in range(4)]

    k.set_vertical_kernel("cuda")
    base = tendency_error()
    k.set_vertical_kernels(inv, fwd)
    assert k.vertical_kernels() == (inv, fwd)
    err = tendency_error()
    assert k.device_status() == 0
    print(f"mixed 128x128x65 vertical ({inv}, {fwd}): tendency errors {err}, dense {base}")
    for a, b in zip(err, base):
        assert a <= 3.0 * b + 1e-7
    rng = np.random.default_rng(4)
    Fb = [torch.from_numpy(rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape)).cuda() for x in dev]
    exact_vjp = [x.cpu().numpy() for x in k64.flux_vjp(777.0, 5.0, *dev, *Fb)]
    got = [x.cpu().numpy() for x in k.flux_vjp(777.0, 5.0, *dev, *Fb)]
    assert max(rel_err(g, e) for g, e in zip(got, exact_vjp)) <= 1e-3
    k.close()
    k64.close()

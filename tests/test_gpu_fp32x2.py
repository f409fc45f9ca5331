"""FP32X2 handles: the xy transforms, quadratic products and vertical
contractions in paired FP32 (float-float) on the FP32 pipe.  The reference has
no such form; its accuracy is checked against the reference's own FP64 outputs
(golden fixtures) and against FP64 handles on the same inputs, with gates far
below the mixed form's: the flux within 1e-9 of max |F|, field tendencies and
states after many RK4 steps within 1e-8 (the metric's bound is 1e-6)."""
import math

import numpy as np
import pytest

from _cases import config_from_case, golden_cases, load_golden, rel_err, rk23_run, state_components_close

pytestmark = pytest.mark.gpu

CASES = golden_cases()
FP32X2_TOL = 1e-9


@pytest.fixture(scope="module")
def wv():
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    wvgpu.load_library()
    return wvgpu


def _conf(wv, c):
    return wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                            planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                            isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32x2_flux_rhs_transforms_and_rk4_match_reference(wv, name):
    cf = CASES[name]
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(_conf(wv, config_from_case(cf)), precision="fp32x2")
    t, t0 = float(g["t"]), float(g["t0"])
    F = k.nonlinearFlux(t, t0, g["Ap"], g["Am"], g["A0"])
    for got, key in zip(F, ("Fp", "Fm", "F0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key, rel_err(got, g[key]))
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    R = k.evaluateRightHandSide(t, t0, g["Ap"], g["Am"], g["A0"])
    for got, key in zip(R, ("Rp", "Rm", "R0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    inv = k.transformWaveVortexToUVWEta(t, t0, g["Ap"], g["Am"], g["A0"])
    assert rel_err(inv, g["inverse"]) <= FP32X2_TOL
    if cf["isHydrostatic"]:
        B = k.transformUVEtaToWaveVortex(g["fields"], t, t0)
    else:
        B = k.transformUVWEtaToWaveVortex(g["fields"], t, t0)
    for got, key in zip(B, ("Bp", "Bm", "B0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    # advection-field entries, derivative bundles and F-grid scalar advection
    args = (t, t0, g["Ap"], g["Am"], g["A0"])
    Fw, adv = k.nonlinearFluxWithAdvectionFields(*args)
    for got, key in zip(Fw, ("with_Fp", "with_Fm", "with_F0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    assert rel_err(adv, g["with_fields"]) <= FP32X2_TOL
    Fu = k.nonlinearFluxUsingAdvectionFields(*args, g["given_fields"])
    for got, key in zip(Fu, ("using_Fp", "using_Fm", "using_F0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    assert rel_err(k.transformWaveVortexToUVW(*args), g["uvw"]) <= FP32X2_TOL
    for q in ((0, 1, 3) if cf["isHydrostatic"] else (0, 1, 2, 3)):
        assert rel_err(k.transformStateFieldDerivatives(*args, q), g[f"deriv_{q}"]) <= FP32X2_TOL, (name, q)
    assert rel_err(k.transformToSpatialDomainWithFAllDerivatives(g["Apm"], g["A0"]), g["fall"]) <= FP32X2_TOL
    assert rel_err(k.transformToSpatialDomainWithGAllDerivatives(g["Apm"], g["A0"]), g["gall"]) <= FP32X2_TOL
    for aa, key in ((False, "scalar_rhs"), (True, "scalar_rhs_aa")):
        assert rel_err(k.advectFGridScalar(g["scalar"], g["given_fields"], aa), g[key]) <= FP32X2_TOL, (name, key)
    Kp, Km, K0, tK = k.rk4(g["rk_Ap"], g["rk_Am"], g["rk_A0"], float(g["rk_t"]), float(g["rk_t0"]), float(g["rk_dt"]),
                           int(g["rk_steps"]))
    assert tK == float(g["rk_tout"])
    assert not state_components_close((Kp, Km, K0), g, ("Kp", "Km", "K0"), FP32X2_TOL), name
    k.close()


def test_fp32x2_single_wave_to_t600(wv):
    """The 16x16x9 single internal wave with adaptive damping, 60 RK4 steps to t = 600 s,
    against the reference's own run."""
    import os
    c = config_from_case(CASES["wave_16x16x9"])
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "wave_16x16x9_t600.npz"))
    k = wv.WVTransformConstantStratificationKernel(_conf(wv, c), precision="fp32x2")
    k.set_forcing(nonlinear=True, adaptive_damping=True)
    Ap, Am, A0, t = k.rk4(g["Ap"], g["Am"], g["A0"], 0.0, 0.0, float(g["dt"]), int(g["steps"]))
    assert t == float(g["t"])
    for a, b in zip((Ap, Am, A0), (g["Kp"], g["Km"], g["K0"])):
        if np.any(b):
            assert rel_err(a, b) <= FP32X2_TOL
    assert rel_err(k.transformWaveVortexToUVWEta(t, 0.0, Ap, Am, A0), g["fields"]) <= FP32X2_TOL
    k.close()


@pytest.mark.parametrize("N,Nz,hydro", [(64, 33, False), (128, 65, False), (96, 49, True)])
def test_fp32x2_fields_after_rk4_steps_match_fp64(wv, N, Nz, hydro):
    """Steep-spectrum turbulent state, 20 RK4 steps at 0.5 x CFL: every field of
    the FP32X2 run within 1e-8 of the FP64 run (relative L2); the flux's field
    tendencies within 1e-8."""
    import torch
    cfg = wv.Configuration(Nx=N, Ny=N, Nz=Nz, Nj=(2 * (Nz - 1)) // 3, Lx=3125.0 * N, Ly=3125.0 * N, Lz=4000.0,
                           latitude=33.0, isHydrostatic=hydro)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
    A = wv.synthetic_state(k64, seed=5, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    fields = [0, 1, 3] if hydro else [0, 1, 2, 3]
    F64 = [x.cpu().numpy() for x in k64.nonlinearFlux(300.0, 0.0, *dev)]
    Fx = [x.cpu().numpy() for x in k.nonlinearFlux(300.0, 0.0, *dev)]
    e64 = k64.transformWaveVortexToUVWEta(0.0, 0.0, *F64)
    ex = k64.transformWaveVortexToUVWEta(0.0, 0.0, *Fx)
    terr = [float(np.linalg.norm(ex[i] - e64[i]) / np.linalg.norm(e64[i])) for i in fields]
    dt = wv.cfl_time_step(k64, *A)
    y64 = [x.clone() for x in dev]
    yx = [x.clone() for x in dev]
    k64.rk4(*y64, 0.0, 0.0, dt, 20)
    k.rk4(*yx, 0.0, 0.0, dt, 20)
    f64 = k64.transformWaveVortexToUVWEta(20 * dt, 0.0, *(x.cpu().numpy() for x in y64))
    fx = k64.transformWaveVortexToUVWEta(20 * dt, 0.0, *(x.cpu().numpy() for x in yx))
    ferr = [float(np.linalg.norm(fx[i] - f64[i]) / np.linalg.norm(f64[i])) for i in fields]
    print(f"{N}x{N}x{Nz} hydro={hydro}: tendency err {terr}, field err after 20 steps {ferr}")
    assert max(terr) <= 1e-8 and max(ferr) <= 1e-8
    k.close()
    k64.close()


def test_fp32x2_rk23_matches_reference_run(wv):
    import torch
    cf, o, ref = rk23_run("odd")
    k = wv.WVTransformConstantStratificationKernel(_conf(wv, config_from_case(cf)), precision="fp32x2")
    rk = wv.WVAdaptiveRK23(k, wv.WVAdaptiveRK23Options(relativeTolerance=o["rtol"], absoluteToleranceScale=o["atol_scale"],
                                                      safetyFactor=o["safety"], rejectionFloorFactor=o["floor"],
                                                      maximumStepFactor=o["max_factor"], maximumStepSize=o["max_step"]))
    y = [torch.from_numpy(np.ascontiguousarray(ref[n])).cuda() for n in ("Ap", "Am", "A0")]
    rk.advanceToTime(*y, ref["t"], ref["t0"], ref["final"], ref["initial"])
    m = rk.metrics()
    assert [m["accepted_steps"], m["rejected_steps"], m["rhs_evaluations"]] == ref["counts"].tolist()[:3]
    for got, want in zip(y, (ref["Kp"], ref["Km"], ref["K0"])):
        assert rel_err(got.cpu().numpy(), want) <= FP32X2_TOL
    rk.close()
    k.close()


@pytest.mark.parametrize("N,Nz,hydro", [(64, 33, False), (128, 65, False), (48, 25, True)])
def test_fp32x2_adjoint_matches_fp64(wv, N, Nz, hydro):
    """The flux VJP and the checkpointed RK4 adjoint of an FP32X2 handle against
    the FP64 handle's on the same state and cotangent (relative 1e-8)."""
    import torch
    cfg = wv.Configuration(Nx=N, Ny=N, Nz=Nz, Nj=(2 * (Nz - 1)) // 3, Lx=3125.0 * N, Ly=3125.0 * N, Lz=4000.0,
                           latitude=33.0, isHydrostatic=hydro)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
    A = wv.synthetic_state(k64, seed=9, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    rng = np.random.default_rng(4)
    cot = [torch.from_numpy(rng.standard_normal(A[0].shape) + 1j * rng.standard_normal(A[0].shape)).cuda() for _ in range(3)]
    g64 = k64.flux_vjp(300.0, 0.0, *dev, *cot)
    gx = k.flux_vjp(300.0, 0.0, *dev, *cot)
    err = [float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(gx, g64)]
    dt = wv.cfl_time_step(k64, *A)
    r64 = k64.rk4_adjoint(*dev, 0.0, 0.0, dt, 6, 3, *cot)
    rx = k.rk4_adjoint(*dev, 0.0, 0.0, dt, 6, 3, *cot)
    rerr = [float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) for a, b in zip(rx, r64)]
    print(f"{N}x{N}x{Nz} hydro={hydro}: flux VJP err {err}, 6-step adjoint err {rerr}")
    assert max(err) <= 1e-8 and max(rerr) <= 1e-8
    k.close()
    k64.close()


def test_fp32x2_tensor_vertical_needs_nj_up_to_96(wv):
    """The digit-sliced tensor-core inverse needs K = Nj / 2 <= 48 per parity
    (shared memory); larger Nj keeps the CUDA-core contraction."""
    k = wv.WVTransformConstantStratificationKernel(
        wv.Configuration(Nx=32, Ny=32, Nz=151, Nj=100, Lx=100e3, Ly=100e3, Lz=4000.0, latitude=33.0), precision="fp32x2")
    with pytest.raises(wv.WVKernelError) as e:
        k.set_vertical_kernel("tensor")
    assert e.value.code == 10
    k.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32x2_tensor_vertical_matches_reference(wv, name):
    """FP32X2 handles with the vertical inverse on the tensor cores (exact
    digit-sliced BF16 GEMMs, k_vinv_tcx): flux, right-hand side, the
    advection-field entries and RK4 against the reference's golden outputs at
    the FP32X2 tolerance; the device status word stays clear."""
    cf = CASES[name]
    g = load_golden(name)
    k = wv.WVTransformConstantStratificationKernel(_conf(wv, config_from_case(cf)), precision="fp32x2")
    k.set_vertical_kernel("tensor")
    t, t0 = float(g["t"]), float(g["t0"])
    args = (t, t0, g["Ap"], g["Am"], g["A0"])
    F = k.nonlinearFlux(*args)
    for got, key in zip(F, ("Fp", "Fm", "F0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key, rel_err(got, g[key]))
    Fw, adv = k.nonlinearFluxWithAdvectionFields(*args)
    for got, key in zip(Fw, ("with_Fp", "with_Fm", "with_F0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    k.set_forcing(nonlinear=True, adaptive_damping=bool(cf["damping"]))
    R = k.evaluateRightHandSide(*args)
    for got, key in zip(R, ("Rp", "Rm", "R0")):
        assert rel_err(got, g[key]) <= FP32X2_TOL, (name, key)
    Kp, Km, K0, tK = k.rk4(g["rk_Ap"], g["rk_Am"], g["rk_A0"], float(g["rk_t"]), float(g["rk_t0"]), float(g["rk_dt"]),
                           int(g["rk_steps"]))
    assert not state_components_close((Kp, Km, K0), g, ("Kp", "Km", "K0"), FP32X2_TOL), name
    assert k.device_status() == 0
    k.close()


@pytest.mark.parametrize("Nx,Ny,Nz,hydro", [(64, 64, 33, False), (48, 40, 24, False), (64, 64, 64, True),
                                            (128, 128, 65, True), (96, 96, 97, False), (256, 256, 129, False)])
def test_fp32x2_tensor_vertical_flux_vs_cuda_cores_and_fp64(wv, Nx, Ny, Nz, hydro):
    """Digit-sliced tensor-core inverse against the CUDA-core paired-FP32
    contraction on 0.1 m/s spectrum states: flux tendencies (u, v, w, eta
    through the FP64 inverse) against the FP64 flux within 1e-9 relative L2,
    and within a small factor of the CUDA-core FP32X2 error."""
    import torch
    import wv_oracle as O
    cfg = wv.Configuration(Nx=Nx, Ny=Ny, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * Nx, Ly=3125.0 * Ny, Lz=4000.0,
                           latitude=33.0, isHydrostatic=hydro)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
    A = wv.synthetic_state(k64, seed=23, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    exact = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in k64.nonlinearFlux(777.0, 5.0, *dev)))
    fields = [0, 1, 3] if hydro else [0, 1, 2, 3]

    def tendency_error(F):
        f = k64.transformWaveVortexToUVWEta(0.0, 0.0, *(x.cpu().numpy() for x in F))
        return [float(np.linalg.norm(f[i] - exact[i]) / np.linalg.norm(exact[i])) for i in fields]

    k.set_vertical_kernel("cuda")
    e_cuda = tendency_error(k.nonlinearFlux(777.0, 5.0, *dev))
    k.set_vertical_kernel("tensor")
    e_tc = tendency_error(k.nonlinearFlux(777.0, 5.0, *dev))
    assert k.device_status() == 0
    print(f"{Nx}x{Ny}x{Nz} hydro={hydro} FP32X2 flux tendency error vs FP64: CUDA cores {e_cuda}, tensor cores {e_tc}")
    for a, b in zip(e_tc, e_cuda):
        assert a <= 1e-9
        assert a <= 20.0 * b + 1e-12
    k.close()
    k64.close()


def test_fp32x2_ensemble_members_equal_single_handles(wv):
    """Member-batched FP32X2 groups in one graph launch step every member exactly
    as a single FP32X2 handle does."""
    import torch
    cfgs = [wv.Configuration(Nx=64, Ny=64, Nz=33, Nj=21, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0),
            wv.Configuration(Nx=48, Ny=40, Nz=25, Nj=16, Lx=150e3, Ly=125e3, Lz=4000.0, latitude=33.0)]
    ens = wv.WVEnsemble(cfgs, [2, 3], precision="fp32x2", autotune=True)
    X, singles = [], []
    for g, cfg in enumerate(cfgs):
        k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
        B = ens.members[g]
        X.append(torch.from_numpy(np.stack([np.stack(wv.synthetic_state(k, seed=60 + 7 * g + m, urms=0.1))
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
        k.close()
    ens.close()


def test_fp32x2_tensor_vertical_members_equal_single_handles(wv):
    """Member-batched FP32X2 groups on the digit-sliced tensor-core inverse (one
    CTA row per member, per-member scratch rows) step every member exactly as a
    single FP32X2 handle on the same kernel does."""
    import torch
    cfgs = [wv.Configuration(Nx=64, Ny=64, Nz=33, Nj=21, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0),
            wv.Configuration(Nx=48, Ny=40, Nz=24, Nj=15, Lx=150e3, Ly=125e3, Lz=4000.0, latitude=33.0)]
    ens = wv.WVEnsemble(cfgs, [3, 2], precision="fp32x2", autotune=False)
    ens.set_vertical_kernel("tensor")
    X, singles = [], []
    for g, cfg in enumerate(cfgs):
        k = wv.WVTransformConstantStratificationKernel(cfg, precision="fp32x2")
        k.set_vertical_kernel("tensor")
        B = ens.members[g]
        X.append(torch.from_numpy(np.stack([np.stack(wv.synthetic_state(k, seed=80 + 7 * g + m, urms=0.1))
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
    ens.close()


@pytest.mark.parametrize("precision,tol", [("fp32x2", 1e-9), ("mixed", 2e-3)])
def test_adjoint_with_tensor_vertical_matches_cuda_cores(wv, precision, tol):
    """The flux VJP and the checkpointed RK4 adjoint (whose forward fluxes keep
    their y spectra for the adjoint x pass) with the tensor-core vertical
    transforms against the same handle on the CUDA-core kernels."""
    import torch
    cfg = wv.Configuration(Nx=64, Ny=64, Nz=33, Nj=21, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
    A = wv.synthetic_state(k, seed=31, urms=0.1)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in A]
    rng = np.random.default_rng(6)
    cot = [torch.from_numpy(rng.standard_normal(A[0].shape) + 1j * rng.standard_normal(A[0].shape)).cuda() for _ in range(3)]
    dt = wv.cfl_time_step(k, *A)
    out = {}
    for kind in ("cuda", "tensor"):
        k.set_vertical_kernel(kind)
        out[kind] = (k.flux_vjp(300.0, 0.0, *dev, *cot), k.rk4_adjoint(*dev, 0.0, 0.0, dt, 6, 3, *cot))
    for a, b in zip(out["tensor"][0] + out["tensor"][1], out["cuda"][0] + out["cuda"][1]):
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) <= tol
    assert k.device_status() == 0
    k.close()


@pytest.mark.parametrize("precision", ["fp32x2", "mixed"])
@pytest.mark.parametrize("N,Nz", [(64, 33), (128, 65), (192, 97), (256, 129)])
def test_fft_variants_match_fp64(wv, precision, N, Nz):
    """Every (y, x) combination of register-line and Stockham FFT kernels
    (wv_set_fft_variants) on FP32X2 and mixed handles: the flux and the flux VJP
    against FP64, each within 3x the default variant's error (the kernels differ
    in rounding order only) and, for FP32X2, the flux within 1e-7 of max |F|
    and the VJP within 1e-8 (single coefficients of high j and small K_h are
    ill-conditioned: FP64's own floor is 3e-10 at 256x256x129, FP32X2 measures
    1e-8 there); the variant reported back is the one asked for (register lines
    exist at these lengths; 192 takes the radix-3 x rows and the 2 x 3 y and
    vertical lines)."""
    import torch
    import wv_oracle as O
    c = O.Config(Nx=N, Ny=N, Nz=Nz, Nj=O.default_nj(Nz), Lx=3125.0 * N, Ly=3125.0 * N, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=13, urms=0.1)
    rng = np.random.default_rng(3)
    Fb = [rng.standard_normal((d.Nkl, c.Nj)) + 1j * rng.standard_normal((d.Nkl, c.Nj)) for _ in range(3)]
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (*A, *Fb)]
    cfg = wv.Configuration(Nx=N, Ny=N, Nz=Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, latitude=33.0)
    k64 = wv.WVTransformConstantStratificationKernel(cfg, precision="fp64")
    F64 = [x.cpu().numpy() for x in k64.nonlinearFlux(777.0, 5.0, *dev[:3])]
    V64 = [x.cpu().numpy() for x in k64.flux_vjp(777.0, 5.0, *dev)]
    k = wv.WVTransformConstantStratificationKernel(cfg, precision=precision)
    assert k.fft_variants() == ("register", "register")
    errs = {}
    for var in (("register", "register"), ("stockham", "stockham"), ("register", "stockham"), ("stockham", "register")):
        k.set_fft_variants(*var)
        assert k.fft_variants() == var
        F = [x.cpu().numpy() for x in k.nonlinearFlux(777.0, 5.0, *dev[:3])]
        V = [x.cpu().numpy() for x in k.flux_vjp(777.0, 5.0, *dev)]
        errs[var] = (max(rel_err(a, b) for a, b in zip(F, F64)), max(rel_err(a, b) for a, b in zip(V, V64)))
        print(f"{precision} {N}x{N}x{Nz} FFT variants {var}: flux {errs[var][0]:.2e}, VJP {errs[var][1]:.2e} against FP64")
    # every variant within 3x of every other (the register lines against the
    # Stockham kernels both ways)
    lo_f = min(e[0] for e in errs.values())
    lo_v = min(e[1] for e in errs.values())
    for var, (ef, ev) in errs.items():
        assert ef <= 3.0 * lo_f + 1e-13 and ev <= 3.0 * lo_v + 1e-13, var
        if precision == "fp32x2":
            assert ef <= 1e-7 and ev <= 1e-8, var
    assert k._lib.wv_set_fft_variants(k._h, 0, 7) != 0  # unknown variant rejected
    assert k.fft_variants() == ("stockham", "register")  # ... and the choice unchanged
    k.close()
    k64.close()

"""The reference-side drop-in (wave-vortex-model_gb300/adapters/WVGPUIntegrationSystem.*):
compiled against the reference's own headers, then stepped by the reference's
own integrators with its right-hand side on the GPU.

  * CPU: the adapter and tests/adapter_driver.cpp compile with -Wall -Werror
    against the reference's CompiledKernel and PortableRuntime headers
    (WVIntegrationContracts.hpp:33-91, WVKernelTypes.hpp) and link against the
    reference build (oracle/_ref/libwvref.so) and libwvgpu.so.
  * GPU: WVIntegrationSystem::evaluateRightHandSide through the adapter equals
    wv_evaluate_rhs bit for bit and the reference's own right-hand side at the
    1e-12 gate; the reference's WVFixedStepRK4::step (PortableRuntime/src/
    WVRungeKutta.cpp:335-462) stepping the GPU system matches wv_rk4_steps and the
    reference's all-CPU run at 1e-12 at the golden grids, and its increments at
    128x128x65 within 3x the flux's measured FP64 floor; the
    reference's WVAdaptiveRK23 (WVRungeKutta.cpp:554-983) stepping the GPU
    system reproduces the reference's own run: accepted / rejected / evaluation
    counts, tolerance hashes (from wv_error_tolerances) and end state.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import ref_lib as R
import wv_oracle as O
from _cases import FP64_REL_TOL, golden_cases, load_golden, parity_tolerance, rel_err, rk23_run, state_components_close

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "wave-vortex-model_gb300", "adapters")
DRIVER = os.path.join(ROOT, "tests", "adapter_driver.cpp")
OUT = os.path.join(ROOT, "oracle", "_ref", "libwvadapter.so")
WVGPU_DIR = os.path.join(ROOT, "wave-vortex-model_gb300", "wvgpu")


def build_adapter():
    """Compiles the adapter and the driver into oracle/_ref/libwvadapter.so."""
    if not R.available():
        pytest.skip("reference C++ not built here: neither a reference checkout nor a staged copy")
    from wvgpu import build
    build.build()
    src = os.path.join(ROOT, "oracle", "_ref", "src")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + ADAPTER,
           "-I" + os.path.join(src, "CompiledKernel", "include"), "-I" + os.path.join(src, "PortableRuntime", "include"),
           "-I" + os.path.join(src, "PortableRuntime", "third_party")]
    sources = [os.path.join(ADAPTER, "WVGPUIntegrationSystem.cpp"), DRIVER]
    deps = sources + [os.path.join(ADAPTER, "WVGPUIntegrationSystem.hpp"), R.LIB, os.path.join(WVGPU_DIR, "libwvgpu.so")]
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(p) for p in deps):
        return OUT
    tmp = OUT + ".tmp"
    cmd = (["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-Werror", "-pthread"] + inc + sources +
           ["-L" + os.path.dirname(R.LIB), "-lwvref", "-L" + WVGPU_DIR, "-lwvgpu",
            "-Wl,-rpath," + os.path.dirname(R.LIB) + ":" + WVGPU_DIR, "-o", tmp])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    os.replace(tmp, OUT)
    return OUT


def test_adapter_compiles_against_reference_headers():
    assert os.path.exists(build_adapter())


# ---- GPU ----------------------------------------------------------------------------


class Adapter:
    """ctypes binding of the driver: one WVGPUIntegrationSystem."""

    def __init__(self, lib, case, precision=0):
        self.lib = lib
        b = dict(R.BASE, **{k: case[k] for k in R.BASE if k in case})
        sizes = (ctypes.c_uint64 * 4)(case["Nx"], case["Ny"], case["Nz"], case["Nj"])
        values = (ctypes.c_double * 9)(case["Lx"], case["Ly"], case["Lz"], b["N0"], b["rho0"], b["g"],
                                       b["planetaryRadius"], b["rotationRate"], case["latitude"])
        flags = (ctypes.c_uint8 * 2)(int(case["isHydrostatic"]), int(case["shouldAntialias"]))
        self.h = ctypes.c_void_p()
        rc = lib.wvad_create(sizes, values, flags, 1 if case.get("damping") else 0, precision, ctypes.byref(self.h))
        assert rc == 0, rc
        self.case = case

    def close(self):
        self.lib.wvad_destroy(self.h)

    def check(self, rc):
        assert rc == 0, self.lib.wvad_message(self.h).decode()

    def rhs(self, Ap, Am, A0, t, t0):
        F = [np.zeros_like(Ap) for _ in range(3)]
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvad_rhs(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0), *map(P, F)))
        return F

    def rk4(self, Ap, Am, A0, t, t0, dt, steps):
        Y = [np.array(a, dtype=np.complex128, copy=True) for a in (Ap, Am, A0)]
        tt = ctypes.c_double(t)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvad_rk4(self.h, *map(P, Y), ctypes.byref(tt), ctypes.c_double(t0), ctypes.c_double(dt),
                                     ctypes.c_int(steps)))
        return Y + [tt.value]

    def rk23(self, Ap, Am, A0, t, t0, final, initial, opts):
        Y = [np.array(a, dtype=np.complex128, copy=True) for a in (Ap, Am, A0)]
        tt = ctypes.c_double(t)
        counts = (ctypes.c_ulonglong * 4)()
        hashes = (ctypes.c_ulonglong * 4)()
        nxt = ctypes.c_double()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvad_rk23(self.h, (ctypes.c_double * 6)(*opts), *map(P, Y), ctypes.byref(tt),
                                      ctypes.c_double(t0), ctypes.c_double(final), ctypes.c_double(initial), counts,
                                      ctypes.byref(nxt), hashes))
        return Y, tt.value, list(counts), list(hashes), nxt.value


@pytest.fixture(scope="module")
def adapter_lib():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    lib = ctypes.CDLL(build_adapter())
    lib.wvad_message.restype = ctypes.c_char_p
    lib.wvad_rhs_evaluations.restype = ctypes.c_uint64
    return lib


def _wv_config(wv, case):
    c = O.Config(**{k: case[k] for k in ("Nx", "Ny", "Nz", "Nj", "Lx", "Ly", "Lz", "latitude", "isHydrostatic",
                                         "shouldAntialias")},
                 **{k: case[k] for k in R.BASE if k in case})
    return c, wv.Configuration(Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, rho0=c.rho0, g=c.g,
                               planetaryRadius=c.planetaryRadius, rotationRate=c.rotationRate, latitude=c.latitude,
                               isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["wave_16x16x9", "hydro_damp_12x10x11", "odd_15x13x9"])
def test_reference_rk4_steps_the_gpu_system(adapter_lib, name):
    import wvgpu
    case = dict(golden_cases()[name])
    g = load_golden(name)
    ad = Adapter(adapter_lib, case)
    t, t0, dt = float(g["t"]), float(g["t0"]), float(case["dt"])
    # the right-hand side through WVIntegrationSystem equals the C ABI's and the reference's
    F = ad.rhs(g["Ap"], g["Am"], g["A0"], t, t0)
    c, cfg = _wv_config(wvgpu, case)
    k = wvgpu.WVTransformConstantStratificationKernel(cfg)
    k.set_forcing(nonlinear=True, adaptive_damping=bool(case["damping"]))
    G = k.evaluateRightHandSide(t, t0, g["Ap"], g["Am"], g["A0"])
    for a, b, key in zip(F, G, ("Rp", "Rm", "R0")):
        assert np.array_equal(a, b)
        assert rel_err(a, g[key]) <= FP64_REL_TOL, key
    # the reference's WVFixedStepRK4 over the GPU system
    Kp, Km, K0, tk = ad.rk4(g["Ap"], g["Am"], g["A0"], t, t0, dt, 2)
    Gp, Gm, G0, tg = k.rk4(g["Ap"], g["Am"], g["A0"], t, t0, dt, 2)
    ref = R.Ref(R.load_lib(), case, R.ENGINE_DIRECT)
    Rp, Rm, R0, tr = ref.rk4(g["Ap"], g["Am"], g["A0"], t, t0, dt, 2)
    assert tk == tg == tr
    for a, b, c_ in zip((Kp, Km, K0), (Gp, Gm, G0), (Rp, Rm, R0)):
        assert rel_err(a, b) <= FP64_REL_TOL
        assert rel_err(a, c_) <= FP64_REL_TOL
    assert adapter_lib.wvad_rhs_evaluations(ad.h) == 1 + 2 * 4
    ad.close()
    k.close()


@pytest.mark.gpu
def test_reference_rk4_steps_the_gpu_system_at_128(adapter_lib):
    """128x128x65 (400 km, the adjoint workload's grid), benchmark spectrum state,
    two WVFixedStepRK4 steps of the GPU system against the reference's all-CPU
    steps (oracle FFT engine)."""
    case = dict(Nx=128, Ny=128, Nz=65, Nj=42, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0, isHydrostatic=False,
                shouldAntialias=True, damping=False)
    c = O.Config(Nx=128, Ny=128, Nz=65, Nj=42, Lx=400e3, Ly=400e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=1, urms=0.1)
    dt = O.cfl_time_step(d, *A)
    ad = Adapter(adapter_lib, case)
    Kp, Km, K0, tk = ad.rk4(*A, 0.0, 0.0, dt, 2)
    ref = R.Ref(R.load_lib(), case, R.ENGINE_ORACLE_FFT)
    Rp, Rm, R0, tr = ref.rk4(*A, 0.0, 0.0, dt, 2)
    assert tk == tr
    # the increments carry the flux's FP64 floor on this steep-spectrum state
    # (two valid FP64 orderings of the flux differ by ~2e-11 here; see
    # tests/test_gpu_reference_cpp.py)
    _, floors = O.noise_floor(O.nonlinear_flux, d, *A, 0.0, 0.0)
    for a, b, a0, fl in zip((Kp, Km, K0), (Rp, Rm, R0), A, floors):
        assert rel_err(a - a0, b - a0) <= parity_tolerance(fl), (rel_err(a - a0, b - a0), fl)
    ad.close()


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["odd", "wave", "hd"])
def test_reference_rk23_steps_the_gpu_system(adapter_lib, key):
    """WVAdaptiveRK23 of the reference over the GPU system: the same counts and
    tolerance hashes as the reference's own run (tests/golden/rk23.npz)."""
    cf, options, run = rk23_run(key)
    ad = Adapter(adapter_lib, dict(cf))
    opts = [options[n] for n in ("rtol", "atol_scale", "safety", "floor", "max_factor", "max_step")]
    Y, t, counts, hashes, nxt = ad.rk23(run["Ap"], run["Am"], run["A0"], run["t"], run["t0"], run["final"],
                                        run["initial"], opts)
    assert counts == [int(x) for x in run["counts"]]
    assert hashes == [int(x) for x in run["hashes"]]
    assert t == run["tout"]
    # components that are pure accumulated rounding (the single wave's A0) gated
    # relative to the state, as for the GPU's own RK23 (tests/test_gpu_rk23.py)
    assert not state_components_close(Y, run, ("Kp", "Km", "K0"), 1e-11)
    ad.close()

"""The oracle's O(N log N) FFT engine (oracle/wv_fft_engine.cpp) inside the
reference's own C++ kernel and runtime, against the same code with the
reference's exact direct-DFT engine (CompiledKernel/adapters/reference/
WVReferenceFFTEngine.cpp:47-107) and against the committed golden fixtures.

The engine is what lets the reference's C++ run at the benchmark grids, so it
is pinned here on every plan the kernel creates: the 2-D r2c/c2r plans with 1,
3 and 4 fields and the REDFT00/RODFT00 plans over 1-3 channels (forward,
inverse, flux, scheduled right-hand side and WVFixedStepRK4 use them all), on
even, odd and prime lengths (Nx = 15, Ny = 13, 9; vertical lines of 2(Nz-1) =
12, 14, 16, 20 points).
"""
import numpy as np
import pytest

import ref_lib as R
from _cases import FP64_REL_TOL, golden_cases, load_golden, rel_err

CASES = golden_cases()
# Extra grids: Nz = 8 puts a radix-7 stage on the vertical lines, Ny = 9 a radix-3 y pass.
EXTRA = {"prime_12x9x8": dict(Nx=12, Ny=9, Nz=8, Nj=4, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0,
                              isHydrostatic=False, shouldAntialias=True, damping=True)}


@pytest.fixture(scope="module")
def lib():
    if not R.available():
        pytest.skip("reference C++ not built here: neither a reference checkout nor a staged copy")
    return R.load_lib()


def _state(shape, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [1e-3 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) for _ in range(3)]


@pytest.mark.parametrize("name", sorted(CASES) + sorted(EXTRA))
def test_engine_matches_direct_dft(lib, name):
    case = dict(CASES.get(name) or EXTRA[name])
    a = R.Ref(lib, case, R.ENGINE_DIRECT)
    b = R.Ref(lib, case, R.ENGINE_ORACLE_FFT)
    Ap, Am, A0 = _state((a.Nkl, case["Nj"]), 11)
    t, t0 = 137.5, -12.25
    nch = 3 if case["isHydrostatic"] else 4
    fields = np.random.default_rng(4).standard_normal((nch, case["Nz"], case["Ny"], case["Nx"])) * 0.05
    # Linear transforms: the engine's own rounding, ~1e-15 relative.
    for x, y in zip(b.forward(fields, t, t0), a.forward(fields, t, t0)):
        assert rel_err(x, y) <= 1e-13
    assert rel_err(b.inverse(Ap, Am, A0, t, t0), a.inverse(Ap, Am, A0, t, t0)) <= 1e-13
    # Flux, scheduled RHS and RK4 chain 19 transforms through the quadratic
    # products and the projection: the reference's own 1e-12 compiled-backend gate.
    for x, y in zip(b.flux(Ap, Am, A0, t, t0), a.flux(Ap, Am, A0, t, t0)):
        assert rel_err(x, y) <= FP64_REL_TOL
    for x, y in zip(b.flux(Ap, Am, A0, t, t0, scheduled=True), a.flux(Ap, Am, A0, t, t0, scheduled=True)):
        assert rel_err(x, y) <= FP64_REL_TOL
    for x, y in zip(b.rk4(Ap, Am, A0, t, t0, 10.0, 2)[:3], a.rk4(Ap, Am, A0, t, t0, 10.0, 2)[:3]):
        assert rel_err(x, y) <= FP64_REL_TOL


@pytest.mark.parametrize("name", sorted(CASES))
def test_engine_reproduces_golden_fixtures(lib, name):
    """The golden fixtures were made with the direct engine; the fast engine
    reproduces them within the reference's 1e-12 gate."""
    case = dict(CASES[name])
    g = load_golden(name)
    b = R.Ref(lib, case, R.ENGINE_ORACLE_FFT)
    t, t0 = float(g["t"]), float(g["t0"])
    for x, key in zip(b.flux(g["Ap"], g["Am"], g["A0"], t, t0), ("Fp", "Fm", "F0")):
        assert rel_err(x, g[key]) <= FP64_REL_TOL, key


def test_engine_threads_reported(lib):
    assert lib.wvref_oracle_fft_threads() >= 1

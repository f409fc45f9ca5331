"""The reference's analytic three-wave triad (UnitTests/TestNonlinearFlux.m:68-262,
testNonlinearWaveTriad): known answers for the energy flux of each wave of a
resonant triad, independent of any FP64 evaluation order.

Setting (TestNonlinearFlux.m:241-243): constant stratification N0 = 5.2e-3,
4 km x 4 km x 2 km (Lx = Ly = 2 Lz, which the analytic expressions assume),
16 x 16 x 9, no transform-level antialiasing, latitude 33 (the transform's
default), hydrostatic and nonhydrostatic.  Three waves, each sign +1, phase 0:
A = (kMode 1, lMode 0, j 1), B = (1, 1, 1), C = (0, 1, 2).  The expected
energy fluxes E_A, E_B, E_C (TestNonlinearFlux.m:229-240) are written in the
waves' own amplitudes, periods and equivalent depths; the energy flux is
2 TE_factor Re(Fp conj(Ap)) (energyFluxFromNonlinearFlux.m:37-44).  Tolerances
are the reference's: AbsTol 1e-15 or RelTol 1e-7 (MATLAB verifyEqual passes
when either holds).

The oracle (numpy restatement) is checked here on the CPU; the GPU's FP64 and
paired-FP32 fluxes in the gpu-marked test.
"""
import math

import numpy as np
import pytest

import wv_oracle as O

ABS_TOL = 1e-15
REL_TOL = 1e-7
U = 0.05  # wave speed amplitude of each triad member (m/s)


def triad_config(hydrostatic):
    return O.Config(Nx=16, Ny=16, Nz=9, Nj=O.default_nj(9), Lx=4e3, Ly=4e3, Lz=2e3, N0=5.2e-3, latitude=33.0,
                    isHydrostatic=hydrostatic, shouldAntialias=False)


def _index(d, kMode, lMode):
    hit = np.nonzero((d.kMode == kMode) & (d.lMode == lMode))[0]
    assert hit.size == 1, (kMode, lMode)
    return int(hit[0])


def triad_state(d):
    """Ap of the three waves (each set to U / (2 |F wave scale|), the amplitude
    initWithWaveModes gives a single wave of speed U); Am = A0 = 0."""
    shape = (d.Nkl, d.c.Nj)
    Ap = np.zeros(shape, np.complex128)
    fws = d.arrays["fWaveScale"] if "fWaveScale" in d.arrays else d.fWaveScale
    idx = {}
    for name, (k, l, j) in {"A": (1, 0, 1), "B": (1, 1, 1), "C": (0, 1, 2)}.items():
        i = _index(d, k, l)
        Ap[i, j] = U / (2.0 * abs(np.asarray(fws).reshape(shape)[i, j]))
        idx[name] = (i, j)
    return (Ap, np.zeros(shape, np.complex128), np.zeros(shape, np.complex128)), idx


def expected_energy_fluxes(d, Ap, idx):
    """E_A, E_B, E_C of TestNonlinearFlux.m:229-240 from the waves' amplitudes."""
    c = d.c
    g, N0, f, Lz = c.g, c.N0, d.f, c.Lz
    L = c.Lx / 2.0 / math.pi
    omega = np.asarray(d.arrays["omega"]).reshape(Ap.shape)
    hpm = np.asarray(d.hpm)
    if c.isHydrostatic:
        Aw = math.sqrt(2.0 * g / Lz) / N0
        ha, hb, hc = hpm[0, 1], hpm[0, 1], hpm[0, 2]
    else:
        Aw = math.sqrt(2.0 * g / ((N0 ** 2 - f ** 2) * Lz))
        ha, hb, hc = (hpm[idx[n]] for n in "ABC")
    N2 = N0 ** 2 / f ** 2
    Ta, Tb, Tc = (f / omega[idx[n]] for n in "ABC")
    A = 2.0 * Ap[idx["A"]] * ha * Aw
    B = 2.0 * Ap[idx["B"]] * hb * Aw / math.sqrt(2.0)
    C = 2.0 * Ap[idx["C"]] * hc * Aw
    s = -math.pi * (A * B * C / 16.0 / L / L / L)
    if c.isHydrostatic:
        E = (s * (7 * Ta + Tb - 8 * Tc + (5 * N2 - 2) * Ta * Tb * Tc),
             s * (-3 * Ta + 3 * Tb + 6 * Tc - 6 * N2 * Ta * Tb * Tc),
             s * (-4 * Ta - 4 * Tb + 2 * Tc + (N2 + 2) * Ta * Tb * Tc))
    else:
        E = (s * (7 * Ta - 4 * Tc + (5 * N2 - 2) * Ta * Tb * Tc),
             s * (-5 * Ta + 3 * Tb + 2 * Tc - 6 * N2 * Ta * Tb * Tc),
             s * (-2 * Ta - 3 * Tb + 2 * Tc + (N2 + 2) * Ta * Tb * Tc))
    return [complex(e).real for e in E]


def check_triad(d, state, idx, flux):
    Ep, _, _ = O.energy_flux(d, *state, *flux)
    expected = expected_energy_fluxes(d, state[0], idx)
    for name, e in zip("ABC", expected):
        got = float(Ep[idx[name]])
        err = abs(got - e)
        assert err <= ABS_TOL or err <= REL_TOL * abs(e), (name, got, e, err / abs(e))
    return expected


@pytest.mark.parametrize("hydrostatic", [False, True])
def test_oracle_triad_energy_fluxes(hydrostatic):
    d = O.build_descriptor(triad_config(hydrostatic))
    state, idx = triad_state(d)
    expected = check_triad(d, state, idx, O.nonlinear_flux(d, *state, 0.0, 0.0))
    assert all(abs(e) > 0 for e in expected)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32x2"])
@pytest.mark.parametrize("hydrostatic", [False, True])
def test_gpu_triad_energy_fluxes(hydrostatic, precision):
    import torch
    import wvgpu
    from wvgpu import build
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build.build()
    c = triad_config(hydrostatic)
    d = O.build_descriptor(c)
    state, idx = triad_state(d)
    k = wvgpu.WVTransformConstantStratificationKernel(wvgpu.Configuration(
        Nx=c.Nx, Ny=c.Ny, Nz=c.Nz, Nj=c.Nj, Lx=c.Lx, Ly=c.Ly, Lz=c.Lz, N0=c.N0, latitude=c.latitude,
        isHydrostatic=c.isHydrostatic, shouldAntialias=c.shouldAntialias), precision=precision)
    check_triad(d, state, idx, k.nonlinearFlux(0.0, 0.0, *state))
    k.close()

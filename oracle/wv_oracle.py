"""CPU oracle for the constant-stratification spectral time step.

TEST INFRASTRUCTURE ONLY.  This module restates, in numpy/scipy, the reference
algorithm of WaveVortexModel's compiled kernel so that tests, the smoke check
and the CPU baseline of the benchmark can check the GPU path against it.  The
shipped GPU library never imports or calls this file.

Parity of this restatement is pinned against golden fixtures produced by the
reference's own C++ sources (CompiledKernel + PortableRuntime + the exact
direct-DFT engine), see tests/golden/make_golden.py and
tests/test_oracle_golden.py.

Storage conventions follow the reference:
  * coefficient arrays are column-major [Nj, Nkl] complex (j fastest); here a
    numpy array of shape (Nkl, Nj) complex128 in C order has the same memory.
  * spatial fields are column-major [Nx, Ny, Nz, ch] (x fastest); here shape
    (ch, Nz, Ny, Nx) in C order.

Citations are to files of the reference project.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:  # scipy gives multi-threaded FFTs; numpy is the fallback.
    import scipy.fft as _sfft

    def _rfft2(x, workers):
        return _sfft.rfft2(x, axes=(-2, -1), workers=workers)

    def _irfft2(x, s, workers):
        return _sfft.irfft2(x, s=s, axes=(-2, -1), norm="forward", workers=workers)

    def _dct1(x, axis):
        return _sfft.dct(x, type=1, axis=axis)

    def _dst1(x, axis):
        return _sfft.dst(x, type=1, axis=axis)

except ImportError:  # pragma: no cover
    _sfft = None

    def _rfft2(x, workers):
        return np.fft.rfft2(x, axes=(-2, -1))

    def _irfft2(x, s, workers):
        return np.fft.irfft2(x, s=s, axes=(-2, -1), norm="forward")

    def _dct1(x, axis):
        x = np.moveaxis(x, axis, -1)
        n = x.shape[-1]
        k = np.arange(n)
        C = 2.0 * np.cos(np.pi * np.outer(k, k) / (n - 1))
        C[:, 0] = 1.0
        C[:, -1] = (-1.0) ** k
        return np.moveaxis(x @ C.T, -1, axis)

    def _dst1(x, axis):
        x = np.moveaxis(x, axis, -1)
        n = x.shape[-1]
        k = np.arange(1, n + 1)
        S = 2.0 * np.sin(np.pi * np.outer(k, k) / (n + 1))
        return np.moveaxis(x @ S.T, -1, axis)


PI = 3.141592653589793238462643383279502884
# WVKernelTypes.cpp:13-16: the F/G normalization uses 9.81 regardless of g.
MODAL_NORMALIZATION_GRAVITY = 9.81
CONTRACT_VERSION = 4  # WVKernelTypes.hpp:11


@dataclass
class Config:
    """WVTransformConstantStratificationConfiguration (WVKernelTypes.hpp:129-146)."""

    Nx: int
    Ny: int
    Nz: int
    Nj: int
    Lx: float
    Ly: float
    Lz: float
    N0: float = 5.2e-3
    rho0: float = 1025.0
    g: float = 9.81
    planetaryRadius: float = 6.371e6
    rotationRate: float = 7.2921e-5
    latitude: float = 33.0
    isHydrostatic: bool = False
    shouldAntialias: bool = True
    contractVersion: int = CONTRACT_VERSION


def default_nj(Nz: int) -> int:
    """Nj = floor(2(Nz-1)/3) (WVGeometryDoublyPeriodicStratifiedConstant.m:61-68)."""
    return (2 * (Nz - 1)) // 3


class OracleError(ValueError):
    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


# WVKernelStatusCode (WVKernelTypes.hpp:22-35)
SUCCESS, INVALID_CONFIGURATION, INVALID_SHAPE, INVALID_POINTER, OVERLAPPING, SIZE_OVERFLOW, \
    ALLOCATION_FAILURE, FFT_PLAN_FAILURE, FFT_EXECUTION_FAILURE, NUMERICAL_FAILURE, UNSUPPORTED, \
    REENTRANT = range(12)


def _dft_modes(n):
    """dftModes (WVKernelTypes.cpp:38-45)."""
    pos = (n + 1) // 2
    return list(range(pos)) + [-v for v in range(n // 2, 0, -1)]


def _dft_index(mode, n):
    return mode if mode >= 0 else n + mode


@dataclass
class Descriptor:
    """Immutable descriptor (WVTransformConstantStratificationDescriptor::create,
    WVKernelTypes.cpp:119-330)."""

    c: Config
    kMode: np.ndarray = None
    lMode: np.ndarray = None
    k: np.ndarray = None
    l: np.ndarray = None
    Kh: np.ndarray = None
    cosAlpha: np.ndarray = None
    sinAlpha: np.ndarray = None
    f: float = 0.0
    z: np.ndarray = None
    m: np.ndarray = None
    h0: np.ndarray = None
    Fg: np.ndarray = None
    Gg: np.ndarray = None
    gWaveScale: np.ndarray = None
    inertialScale: np.ndarray = None
    apmWProjectionPrefactor: np.ndarray = None
    hpm: np.ndarray = None
    arrays: dict = field(default_factory=dict)
    NxHalf: int = 0
    storageRow: np.ndarray = None
    conjugated: np.ndarray = None
    completionRows: np.ndarray = None
    completionSources: np.ndarray = None
    selfConjugateRows: np.ndarray = None

    @property
    def Nkl(self):
        return len(self.kMode)

    @property
    def M(self):
        return self.Nkl * self.c.Nj


def build_descriptor(c: Config) -> Descriptor:
    if c.contractVersion != CONTRACT_VERSION:
        raise OracleError(INVALID_CONFIGURATION, "Unsupported kernel contract version.")
    if c.Nx < 2 or c.Ny < 2 or c.Nz < 3 or c.Nj < 1 or c.Nj > c.Nz - 1:
        raise OracleError(INVALID_CONFIGURATION,
                          "Nx and Ny must be at least 2, Nz at least 3, and Nj must lie in [1,Nz-1].")
    for v in (c.Lx, c.Ly, c.Lz, c.N0, c.rho0, c.g, c.planetaryRadius, c.rotationRate):
        if not (math.isfinite(v) and v > 0.0):
            raise OracleError(INVALID_CONFIGURATION,
                              "Physical lengths and constants must be finite and positive, and latitude must lie in [-90,90].")
    if not math.isfinite(c.latitude) or abs(c.latitude) > 90.0:
        raise OracleError(INVALID_CONFIGURATION,
                          "Physical lengths and constants must be finite and positive, and latitude must lie in [-90,90].")
    d = Descriptor(c=c)
    Nx, Ny, Nz, Nj = c.Nx, c.Ny, c.Nz, c.Nj
    kModes = _dft_modes(Nx)
    lModes = _dft_modes(Ny)
    maxAbsK = 2.0 * PI * (float(Nx // 2) / c.Lx)
    K, L = [], []
    # WVKernelTypes.cpp:143-158: l outer, k inner; primary, non-Nyquist, inside 2/3 disk.
    for lm in lModes:
        for km in kModes:
            kSelf = km == 0 or (Nx % 2 == 0 and km == -(Nx // 2))
            lSelf = lm == 0 or (Ny % 2 == 0 and lm == -(Ny // 2))
            primary = lm > 0 or (lSelf and (km > 0 or kSelf))
            nyq = (Nx % 2 == 0 and km == -(Nx // 2)) or (Ny % 2 == 0 and lm == -(Ny // 2))
            if not primary or nyq:
                continue
            K.append(km)
            L.append(lm)
    K = np.array(K, dtype=np.int64)
    L = np.array(L, dtype=np.int64)
    k = 2.0 * PI * (K.astype(np.float64) / c.Lx)
    l = 2.0 * PI * (L.astype(np.float64) / c.Ly)
    # radialMagnitude: sqrt(k*k + l*l) with no fused multiply-add (WVKernelTypes.cpp:22-29)
    Kh = np.sqrt(k * k + l * l)
    if c.shouldAntialias:
        keep = ~(Kh > 2.0 * maxAbsK / 3.0)
        K, L, k, l, Kh = K[keep], L[keep], k[keep], l[keep], Kh[keep]
    order = np.lexsort((L, K, Kh))  # sort by (Kh, kMode, lMode) (WVKernelTypes.cpp:159-166)
    K, L, k, l, Kh = K[order], L[order], k[order], l[order], Kh[order]
    d.kMode, d.lMode, d.k, d.l, d.Kh = K, L, k, l, Kh
    with np.errstate(divide="ignore", invalid="ignore"):
        d.cosAlpha = np.where(Kh == 0.0, 0.0, k / Kh)
        d.sinAlpha = np.where(Kh == 0.0, 0.0, l / Kh)

    f = 2.0 * c.rotationRate * math.sin(c.latitude * PI / 180.0)
    d.f = f
    dz = c.Lz / float(Nz - 1)
    d.z = dz * np.arange(Nz, dtype=np.float64) - c.Lz
    jj = np.arange(Nj, dtype=np.float64)
    m = jj * PI / c.Lz
    d.m = m
    h0 = np.empty(Nj)
    h0[0] = c.Lz
    h0[1:] = c.N0 * c.N0 / (c.g * m[1:] * m[1:])
    d.h0 = h0
    N02 = c.N0 * c.N0
    f2 = f * f
    if not c.isHydrostatic and N02 <= f2:
        raise OracleError(INVALID_CONFIGURATION,
                          "Nonhydrostatic constant stratification requires N0 squared greater than f squared.")
    sign = np.where(np.arange(Nj) % 2 == 0, 1.0, -1.0)
    root = math.sqrt(2.0 * MODAL_NORMALIZATION_GRAVITY / (c.Lz * N02))
    rootw = math.sqrt(2.0 * MODAL_NORMALIZATION_GRAVITY / (c.Lz * (N02 - f2))) if N02 != f2 else float("inf")
    Fg = sign * h0 * m * root
    Fg[0] = 2.0
    Gg = sign * root
    Gg[0] = 1.0
    if c.isHydrostatic:
        Gw_v = Gg.copy()
    else:
        Gw_v = sign * rootw
        Gw_v[0] = Gg[0]
    Gwg_v = Gg / Gw_v
    d.Fg, d.Gg = Fg, Gg
    d.gWaveScale = Gg / Gwg_v

    # Per-coefficient arrays (WVKernelTypes.cpp:214-284), shape (Nkl, Nj).
    KhC = Kh[:, None]
    Kh2 = KhC * KhC
    full = (len(Kh), Nj)
    M_ = m[None, :]
    signC = sign[None, :]
    jC = np.arange(Nj)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        if c.isHydrostatic:
            hpm = np.broadcast_to(N02 / (c.g * M_ * M_), full).copy()
        else:
            hpm = (N02 - f2) / (c.g * (M_ * M_ + Kh2))
        hpm[:, 0] = 1.0
        FgC = Fg[None, :]
        GgC = Gg[None, :]
        if c.isHydrostatic:
            Fw = np.broadcast_to(FgC, full).copy()
            Gw = np.broadcast_to(GgC, full).copy()
        else:
            Fw = signC * hpm * M_ * rootw
            Gw = np.broadcast_to(signC * rootw, full).copy()
            Fw[:, 0] = 2.0
            Gw[:, 0] = 1.0
        omega = np.sqrt(c.g * hpm * Kh2 + f2)
        Fwg = FgC / Fw
        Gwg = GgC / Gw
        fWaveScale = FgC / Fwg
        inertialScale = (0.5 * Fwg / FgC)[0]
        prefactor = sign * math.sqrt(c.g * c.Lz / (2.0 * (N02 - f2))) if N02 != f2 else sign * float("inf")
        ApmDScaled = np.broadcast_to((m / 2.0) * prefactor, full).copy()
        isWave = (KhC > 0.0) & (jC > 0)
        isInertial = np.broadcast_to(KhC == 0.0, full)
        isGeo = np.broadcast_to(KhC > 0.0, full)
        isMDA = (KhC == 0.0) & (jC > 0)
        cosA = d.cosAlpha[:, None]
        sinA = d.sinAlpha[:, None]
        kC = k[:, None]
        lC = l[:, None]
        z0 = np.zeros(full)
        gws = d.gWaveScale[None, :]
        UAp_r = np.where(isWave, cosA * fWaveScale, np.where(isInertial, fWaveScale, 0.0))
        UAp_i = np.where(isWave, (-(f / omega) * sinA) * fWaveScale, 0.0)
        VAp_r = np.where(isWave, sinA * fWaveScale, 0.0)
        VAp_i = np.where(isWave, ((f / omega) * cosA) * fWaveScale, np.where(isInertial, fWaveScale, 0.0))
        WAp_i = np.where(isWave, (-KhC * hpm) * gws, 0.0)
        NAp = np.where(isWave, (-KhC * hpm / omega) * gws, 0.0)
        deltaScale = h0[None, :] * Gwg / FgC
        ApmD_i = np.where(isWave, (-1.0 / (2.0 * KhC * hpm)) * deltaScale, 0.0)
        ApmN = np.where(isWave, (-omega / (2.0 * KhC * hpm)) * Gwg / GgC, 0.0)
        Lr2Inverse = np.where(jC == 0, 0.0, f2 / (c.g * h0[None, :]))
        denom = Kh2 + Lr2Inverse
        UA0_i = np.where(isGeo, (lC / denom) * FgC, 0.0)
        VA0_i = np.where(isGeo, (-kC / denom) * FgC, 0.0)
        NA0 = np.where(isGeo, np.where(jC == 0, 0.0, -(f / c.g) / denom) * GgC, np.where(isMDA, GgC, 0.0))
        A0FromVorticity = np.where(isGeo, 1.0 / FgC, np.where(isMDA, (f2 / (2.0 * h0[None, :])) / FgC, 0.0))
        A0FromBuoyancy = np.where(isGeo, np.where(jC == 0, 0.0, (-f / h0[None, :]) / GgC),
                                  np.where(isMDA, 1.0 / GgC, 0.0))
    d.hpm = hpm
    d.inertialScale = inertialScale
    d.apmWProjectionPrefactor = prefactor
    d.arrays = dict(
        omega=omega, fWaveScale=fWaveScale,
        UAp=UAp_r + 1j * UAp_i, VAp=VAp_r + 1j * VAp_i, WAp=z0 + 1j * WAp_i, NAp=NAp,
        UA0=z0 + 1j * UA0_i, VA0=z0 + 1j * VA0_i, NA0=NA0,
        A0FromVorticity=A0FromVorticity, A0FromBuoyancy=A0FromBuoyancy,
        ApmD=z0 + 1j * ApmD_i, ApmN=ApmN, ApmDScaled=ApmDScaled,
    )

    # Half-spectrum mappings (WVKernelTypes.cpp:286-321)
    NxHalf = Nx // 2 + 1
    d.NxHalf = NxHalf
    conj = K < 0
    kk = np.where(conj, -K, K)
    ll = np.where(conj, -L, L)
    ll_idx = np.where(ll >= 0, ll, Ny + ll)
    d.storageRow = (kk + NxHalf * ll_idx).astype(np.int64)
    d.conjugated = conj
    represented = np.zeros(NxHalf * Ny, dtype=bool)
    represented[d.storageRow] = True
    comp_rows, comp_src, self_rows = [], [], []
    for iL in range(Ny):
        lm = iL if iL <= Ny // 2 else iL - Ny
        dest = NxHalf * _dft_index(lm, Ny)
        src = NxHalf * _dft_index(-lm, Ny)
        if not represented[dest] and represented[src]:
            comp_rows.append(dest)
            comp_src.append(src)
        if lm == 0 or (Ny % 2 == 0 and abs(lm) == Ny // 2):
            if represented[dest]:
                self_rows.append(dest)
    d.completionRows = np.array(comp_rows[::-1], dtype=np.int64)
    d.completionSources = np.array(comp_src[::-1], dtype=np.int64)
    d.selfConjugateRows = np.array(self_rows, dtype=np.int64)
    return d


# ---------------------------------------------------------------------------
# Vertical transforms with the reference's plan semantics
# (verticalSpecification, WVTransformConstantStratificationKernel.cpp:161-174;
#  REDFT00/RODFT00 definitions, adapters/reference/WVReferenceFFTEngine.cpp:88-107)


def _dct_inplace_complex(x, axis=-1):
    return _dct1(x.real, axis) + 1j * _dct1(x.imag, axis)


def _dst_positions(x):
    """DST-I over storage positions 1..Nz-2 along the last axis; positions 0 and
    Nz-1 pass through unchanged (in-place plan offset by one)."""
    y = x.copy()
    inner = x[..., 1:-1]
    y[..., 1:-1] = _dst1(inner.real, -1) + 1j * _dst1(inner.imag, -1)
    return y


def _columns_to_half(desc, cols):
    """Scatter per-WV-mode z columns (ch, Nkl, Nz) into the half spectrum
    (ch, Nz, Ny, NxHalf); conjugate where the mode is stored conjugated, then
    Hermitian completion and self-conjugate rows (completeHermitianBoundaries,
    WVTransformConstantStratificationKernel.cpp:433-438)."""
    c = desc.c
    nch = cols.shape[0]
    half = np.zeros((nch, c.Ny * desc.NxHalf, c.Nz), dtype=np.complex128)
    vals = np.where(desc.conjugated[None, :, None], np.conj(cols), cols)
    half[:, desc.storageRow, :] = vals
    if len(desc.completionRows):
        half[:, desc.completionRows, :] = np.conj(half[:, desc.completionSources, :])
    if len(desc.selfConjugateRows):
        half[:, desc.selfConjugateRows, :] = half[:, desc.selfConjugateRows, :].real
    return half


def _half_rows_to_spatial(desc, half_rows):
    """c2r (unnormalized, FFTW semantics) of half spectra stored by row
    (ch, rows, Nz) -> fields (ch, Nz, Ny, Nx)."""
    c = desc.c
    nch = half_rows.shape[0]
    h = half_rows.reshape(nch, c.Ny, desc.NxHalf, c.Nz).transpose(0, 3, 1, 2)
    return _irfft2(h, (c.Ny, c.Nx), -1)


def _spatial_to_half_rows(desc, fields):
    """r2c (unnormalized) of fields (ch, Nz, Ny, Nx) -> (ch, rows, Nz)."""
    c = desc.c
    h = _rfft2(fields, -1)  # (ch, Nz, Ny, NxHalf)
    nch = fields.shape[0]
    return h.transpose(0, 2, 3, 1).reshape(nch, c.Ny * desc.NxHalf, c.Nz)


def _gather_columns(desc, half_rows):
    """Read the stored value of every WV mode (storedValue<Conjugated>,
    WVTransformConstantStratificationKernel.cpp:211-216): (ch, Nkl, Nz)."""
    v = half_rows[:, desc.storageRow, :]
    return np.where(desc.conjugated[None, :, None], np.conj(v), v)


def _pad_z(desc, coef):
    """(…, Nkl, Nj) -> (…, Nkl, Nz) with zeros for j >= Nj."""
    c = desc.c
    out = np.zeros(coef.shape[:-1] + (c.Nz,), dtype=np.complex128)
    out[..., : c.Nj] = coef
    return out


def _forward_dct_columns(desc, cols):
    """DCT-I then normalizeForwardDCT (kernel.cpp:176-183); returns (…, Nkl, Nj)."""
    c = desc.c
    y = _dct_inplace_complex(cols, -1) * (1.0 / float(c.Nz - 1))
    y[..., c.Nz - 1] *= 0.5
    return y[..., : c.Nj]


def _forward_dst_columns(desc, cols):
    """DST-I then normalizeForwardDST (kernel.cpp:185-193)."""
    c = desc.c
    y = _dst_positions(cols)
    y = y * (1.0 / float(c.Nz - 1))
    y[..., 0] = 0.0
    y[..., c.Nz - 1] = 0.0
    return y[..., : c.Nj]


# ---------------------------------------------------------------------------
# Coefficient algebra (WVCoefficientFormulas.hpp)


def phase(desc, t, t0):
    el = t - t0
    return np.cos(desc.arrays["omega"] * el) + 1j * np.sin(desc.arrays["omega"] * el)


def _field_values(desc, Ap, Am, A0, p):
    """coefficientValueForField<0..3> (WVCoefficientFormulas.hpp:27-33) on
    evolved coefficients (evolveWaveVortexCoefficients :23-25)."""
    a = desc.arrays
    Ape = Ap * p
    Ame = Am * np.conj(p)
    u = a["UAp"] * Ape + np.conj(a["UAp"]) * Ame + a["UA0"] * A0
    v = a["VAp"] * Ape + np.conj(a["VAp"]) * Ame + a["VA0"] * A0
    w = a["WAp"] * Ape + a["WAp"] * Ame
    n = Ape * a["NAp"] + Ame * (-a["NAp"]) + A0 * a["NA0"]
    return u, v, w, n


def _inverse_columns_cos(desc, coef):
    return _dct_inplace_complex(_pad_z(desc, coef), -1)


def _inverse_columns_sin(desc, coef):
    return _dst_positions(_pad_z(desc, coef))


def inverse_uvweta(desc, Ap, Am, A0, t, t0):
    """transformWaveVortexToUVWEta (kernel.cpp:745-776): returns (4, Nz, Ny, Nx)."""
    c = desc.c
    p = phase(desc, t, t0)
    u, v, w, n = _field_values(desc, Ap, Am, A0, p)
    u = u * 0.5
    v = v * 0.5
    w = w * 0.5
    n = n * 0.5
    w[:, 0] = 0.0
    n[:, 0] = 0.0
    if c.Nj == c.Nz:  # j + 1 == Nz endpoint (never reached since Nj <= Nz-1)
        w[:, -1] = 0.0
        n[:, -1] = 0.0
    cols = np.stack([_inverse_columns_cos(desc, u), _inverse_columns_cos(desc, v),
                     _inverse_columns_sin(desc, w), _inverse_columns_sin(desc, n)])
    half = _columns_to_half(desc, cols)
    return _half_rows_to_spatial(desc, half)


def velocity_fields(desc, Ap, Am, A0, t, t0):
    """transformWaveVortexToUVWImpl (kernel.cpp:778-805): (3, Nz, Ny, Nx)."""
    p = phase(desc, t, t0)
    u, v, w, _ = _field_values(desc, Ap, Am, A0, p)
    u = u * 0.5
    v = v * 0.5
    w = w * 0.5
    w[:, 0] = 0.0
    cols = np.stack([_inverse_columns_cos(desc, u), _inverse_columns_cos(desc, v), _inverse_columns_sin(desc, w)])
    return _half_rows_to_spatial(desc, _columns_to_half(desc, cols))


def derivative_fields(desc, Ap, Am, A0, t, t0, target):
    """transformToSpatialDomainWithDerivativesFromStateImpl (kernel.cpp:907-945)
    with normalizedDerivativeSpectrum (WVCoefficientFormulas.hpp:42-58):
    returns (3, Nz, Ny, Nx) = d/dx, d/dy, d/dz of field `target`."""
    p = phase(desc, t, t0)
    val = _field_values(desc, Ap, Am, A0, p)[target]
    # Column values are taken in the WV (unconjugated) frame: derivative factors
    # i*k, i*l use the mode's own wavenumbers; conjugated storage then conjugates.
    kC = desc.k[:, None]
    lC = desc.l[:, None]
    mC = desc.m[None, :]
    cosine = target < 2
    x = val * (1j * kC)
    y = val * (1j * lC)
    zz = val * (-mC if cosine else mC)
    if cosine:
        x = x * 0.5
        y = y * 0.5
        zz = zz * 0.5
        zz[:, 0] = 0.0
        cols = np.stack([_inverse_columns_cos(desc, x), _inverse_columns_cos(desc, y), _inverse_columns_sin(desc, zz)])
    else:
        x = x * 0.5
        y = y * 0.5
        x[:, 0] = 0.0
        y[:, 0] = 0.0
        zz = zz * 0.5
        cols = np.stack([_inverse_columns_sin(desc, x), _inverse_columns_sin(desc, y), _inverse_columns_cos(desc, zz)])
    return _half_rows_to_spatial(desc, _columns_to_half(desc, cols))


def _project_target(desc, S, target, p, Fp, Fm, F0):
    """projectSingleFluxTargetImpl + projectFluxTargetMode
    (kernel.cpp:947-990, 396-431). Accumulates in place."""
    c = desc.c
    a = desc.arrays
    half = _spatial_to_half_rows(desc, S[None])
    cols = _gather_columns(desc, half)[0]  # (Nkl, Nz)
    if target < 2:
        coef = _forward_dct_columns(desc, cols)
    else:
        coef = _forward_dst_columns(desc, cols)
    value = coef * (1.0 / float(c.Nx * c.Ny))
    kC = desc.k[:, None]
    lC = desc.l[:, None]
    if target == 0:
        A0c = value * (1j * (-lC)) * a["A0FromVorticity"]
    elif target == 1:
        A0c = value * (1j * kC) * a["A0FromVorticity"]
    elif target == 3:
        A0c = value * a["A0FromBuoyancy"]
    else:
        A0c = np.zeros_like(value)
    buoyV = (value if target == 3 else 0.0) - A0c * a["NA0"]
    buoy = buoyV * a["ApmN"]
    if c.isHydrostatic:
        if target == 0:
            wave = value * (1j * kC) * a["ApmD"]
        elif target == 1:
            wave = value * (1j * lC) * a["ApmD"]
        else:
            wave = np.zeros_like(value)
    else:
        if target == 0:
            wave = value * (desc.cosAlpha[:, None] * a["ApmDScaled"])
        elif target == 1:
            wave = value * (desc.sinAlpha[:, None] * a["ApmDScaled"])
        elif target == 2:
            wave = value * (1j * ((desc.Kh[:, None] / 2.0) * desc.apmWProjectionPrefactor[None, :]))
        else:
            wave = np.zeros_like(value)
    cp = wave + buoy
    cm = wave - buoy
    # inertial override for WV index 0 (inertialCoefficientPair<Target>, WVCoefficientFormulas.hpp:101-107)
    sc = desc.inertialScale
    if target == 0:
        cp[0] = value[0] * sc
    elif target == 1:
        cp[0] = value[0] * (-1j) * sc
    else:
        cp[0] = 0.0
    cm[0] = np.conj(cp[0])
    Fp += cp * np.conj(p)
    Fm += cm * p
    F0 += A0c


def nonlinear_flux(desc, Ap, Am, A0, t, t0, advection=None):
    """nonlinearFluxImpl (kernel.cpp:1173-1244): returns (Fp, Fm, F0).  With
    `advection` (3, Nz, Ny, Nx) given, that velocity advects the state's fields
    (nonlinearFluxUsingAdvectionFields, kernel.cpp:1160-1171)."""
    c = desc.c
    p = phase(desc, t, t0)
    if advection is None:
        U, V, W = velocity_fields(desc, Ap, Am, A0, t, t0)
    else:
        U, V, W = advection
    Fp = np.zeros_like(Ap)
    Fm = np.zeros_like(Ap)
    F0 = np.zeros_like(Ap)
    targets = (0, 1, 3) if c.isHydrostatic else (0, 1, 2, 3)
    for q in targets:
        dx, dy, dz = derivative_fields(desc, Ap, Am, A0, t, t0, q)
        S = -(U * dx + V * dy + W * dz)
        _project_target(desc, S, q, p, Fp, Fm, F0)
    return Fp, Fm, F0


def flux_with_advection(desc, Ap, Am, A0, t, t0):
    """nonlinearFluxWithAdvectionFields (kernel.cpp:1148-1158): (Fp, Fm, F0), (u, v, w)."""
    adv = velocity_fields(desc, Ap, Am, A0, t, t0)
    return nonlinear_flux(desc, Ap, Am, A0, t, t0, advection=adv), adv


def inverse_uvw(desc, Ap, Am, A0, t, t0):
    """transformWaveVortexToUVW (kernel.cpp:696-717): (3, Nz, Ny, Nx)."""
    return velocity_fields(desc, Ap, Am, A0, t, t0)


def family_derivatives(desc, Apm, A0, ffamily):
    """transformToSpatialDomainWith{F,G}AllDerivatives (kernel.cpp:819-863) with
    fieldFamilyDerivativeSpectrum (WVCoefficientFormulas.hpp:60-73): value =
    Apm waveScale + A0 geostrophicScale (F: fWaveScale, Fg; G: gWaveScale, Gg),
    its i k, i l and -m (F) / +m (G) derivatives; F values are cosine-family
    (inverse DCT x 0.5) with a sine-family z derivative (inverse DST x 0.5,
    endpoints 0), G the other way round.  Returns (4, Nz, Ny, Nx)."""
    kC = desc.k[:, None]
    lC = desc.l[:, None]
    mC = desc.m[None, :]
    if ffamily:
        val = Apm * desc.arrays["fWaveScale"] + A0 * desc.Fg[None, :]
    else:
        val = Apm * desc.gWaveScale[None, :] + A0 * desc.Gg[None, :]
    x = val * (1j * kC)
    y = val * (1j * lC)
    zz = val * (-mC if ffamily else mC)
    cos_ = lambda v: _inverse_columns_cos(desc, v * 0.5)
    def sin_(v):
        v = v * 0.5
        v[:, 0] = 0.0
        return _inverse_columns_sin(desc, v)
    if ffamily:
        cols = np.stack([cos_(val), cos_(x), cos_(y), sin_(zz)])
    else:
        cols = np.stack([sin_(val), sin_(x), sin_(y), cos_(zz)])
    return _half_rows_to_spatial(desc, _columns_to_half(desc, cols))


def scalar_wavenumbers(desc):
    """Row wavenumbers of the F-grid scalar pipeline (kernel.cpp:1067-1072): k over
    the NxHalf columns with k = 0 at an even-Nx Nyquist column, l over the Ny rows
    by signed mode index (the even-Ny Nyquist row keeps its negative l)."""
    c = desc.c
    NxHalf = c.Nx // 2 + 1
    kIndex = np.arange(NxHalf)
    k = 2.0 * PI * kIndex / c.Lx
    if c.Nx % 2 == 0:
        k[c.Nx // 2] = 0.0
    lIndex = np.arange(c.Ny)
    lMode = np.where(lIndex < (c.Ny + 1) // 2, lIndex, lIndex - c.Ny)
    l = 2.0 * PI * lMode / c.Ly
    return k, l


def scalar_antialias_rows(desc):
    """Half-spectrum rows kept by the scalar antialias (kernel.cpp:466-471): storage
    rows of every WV mode, their Hermitian completion and source rows."""
    c = desc.c
    keep = np.zeros(c.Ny * (c.Nx // 2 + 1), dtype=bool)
    keep[desc.storageRow] = True
    if len(desc.completionRows):
        keep[desc.completionRows] = True
        keep[desc.completionSources] = True
    return keep


def advect_fgrid_scalar(desc, scalar, advection, antialias):
    """advectFGridScalar (kernel.cpp:1032-1138): -(u ds/dx + v ds/dy + w ds/dz) of
    an F-grid scalar (Nz, Ny, Nx) with spectral derivatives: x, y by the
    half-spectrum r2c/c2r pair; z by forward DCT-I (normalizeForwardDCT), times
    -m_j on the interior modes, normalizeInverseDST and DST-I on the interior
    points; self-conjugate rows real.  With `antialias`, the result is filtered to
    the transform's rows (antialiasScalarInPlace, kernel.cpp:1008-1030)."""
    c = desc.c
    Nz = c.Nz
    NxHalf = c.Nx // 2 + 1
    hs = 1.0 / float(c.Nx * c.Ny)
    k, l = scalar_wavenumbers(desc)
    val = _rfft2(scalar, -1) * hs                          # (Nz, Ny, NxHalf)
    cx = val * (1j * k)[None, None, :]
    cy = val * (1j * l)[None, :, None]
    d = (_dct1(val.real, 0) + 1j * _dct1(val.imag, 0)) * (1.0 / float(Nz - 1))
    d[Nz - 1] *= 0.5
    m = PI * np.arange(Nz) / c.Lz
    d[1:Nz - 1] *= -m[1:Nz - 1, None, None]
    d[0] = 0.0
    d[Nz - 1] = 0.0
    d[1:Nz - 1] *= 0.5
    cz = np.zeros_like(d)
    inner = d[1:Nz - 1]
    cz[1:Nz - 1] = _dst1(inner.real, 0) + 1j * _dst1(inner.imag, 0)
    spec = np.stack([cx, cy, cz])                          # (3, Nz, Ny, NxHalf)
    rows = np.asarray(desc.selfConjugateRows, dtype=np.int64)
    if len(rows):
        ky, kx = rows // NxHalf, rows % NxHalf
        spec[:, :, ky, kx] = spec[:, :, ky, kx].real
    dx, dy, dz = _irfft2(spec, (c.Ny, c.Nx), -1)
    U, V, W = advection
    rhs = -(U * dx + V * dy + W * dz)
    if antialias:
        keep = scalar_antialias_rows(desc).reshape(c.Ny, NxHalf)
        H = _rfft2(rhs, -1) * np.where(keep, hs, 0.0)[None, :, :]
        rhs = _irfft2(H, (c.Ny, c.Nx), -1)
    return rhs


def forward(desc, fields, t, t0):
    """transformUVWEtaToWaveVortexImpl / transformUVEtaToWaveVortexImpl
    (kernel.cpp:651-684, 597-635) with projectNonhydrostaticMode /
    projectHydrostaticMode (:335-370, :299-333). fields: (ch, Nz, Ny, Nx)."""
    c = desc.c
    a = desc.arrays
    half = _spatial_to_half_rows(desc, fields)
    cols = _gather_columns(desc, half)
    hs = 1.0 / float(c.Nx * c.Ny)
    kC = desc.k[:, None]
    lC = desc.l[:, None]
    if c.isHydrostatic:
        U = _forward_dct_columns(desc, cols[0]) * hs
        V = _forward_dct_columns(desc, cols[1]) * hs
        N = _forward_dst_columns(desc, cols[2]) * hs
        W = None
    else:
        U = _forward_dct_columns(desc, cols[0]) * hs
        V = _forward_dct_columns(desc, cols[1]) * hs
        W = _forward_dst_columns(desc, cols[2]) * hs
        N = _forward_dst_columns(desc, cols[3]) * hs
    A0 = (V * (1j * kC) - U * (1j * lC)) * a["A0FromVorticity"] + N * a["A0FromBuoyancy"]
    buoy = (N - A0 * a["NA0"]) * a["ApmN"]
    if c.isHydrostatic:
        div = U * (1j * kC) + V * (1j * lC)
        wave = a["ApmD"] * div
    else:
        delta = (U * desc.cosAlpha[:, None] + V * desc.sinAlpha[:, None]) * a["ApmDScaled"]
        wbar = (1j * ((desc.Kh[:, None] / 2.0) * desc.apmWProjectionPrefactor[None, :])) * W
        wave = delta + wbar
    Ap = wave + buoy
    Am = wave - buoy
    Ap[0] = (U[0] - V[0] * 1j) * desc.inertialScale
    Am[0] = np.conj(Ap[0])
    p = phase(desc, t, t0)
    return Ap * np.conj(p), Am * p, A0


# ---------------------------------------------------------------------------
# Forcing: adaptive damping (PortableRuntime/src/WVForcingEngine.cpp:30-38, 352-381, 710-726)


def _vanishing_filter(value, cutoff, maximum):
    value = abs(value)
    if value < cutoff:
        return 0.0
    if value > maximum:
        return 1.0
    if maximum == cutoff:
        return 1.0 if value >= maximum else 0.0
    ratio = (value - maximum) / (value - cutoff)
    return math.exp(-(ratio * ratio))


def adaptive_damping_operator(desc):
    c = desc.c
    f2 = desc.f * desc.f
    if not f2 > 0.0:
        raise OracleError(UNSUPPORTED, "Adaptive damping requires nonzero Coriolis frequency.")
    maxComp = float(np.max(np.maximum(np.abs(desc.k), np.abs(desc.l))))
    if not maxComp > 0.0:
        raise OracleError(INVALID_CONFIGURATION, "Adaptive damping requires resolved horizontal wavenumbers.")
    effRes = PI / maxComp
    dklMin = min(2.0 * PI / c.Lx, 2.0 * PI / c.Ly)
    klCut = dklMin * (maxComp / dklMin) ** 0.75
    jMax = float(c.Nj - 1)
    jCut = jMax ** 0.75 if c.Nj > 2 else 0.0
    prefXY = effRes / (PI * PI)
    refLr2 = c.g * desc.h0[-1] / f2
    prefZ = (PI * PI * refLr2 / (effRes * effRes)) * prefXY
    damp = np.empty((desc.Nkl, c.Nj))
    for i in range(desc.Nkl):
        Qkl = _vanishing_filter(desc.Kh[i], klCut, maxComp)
        for j in range(c.Nj):
            Qj = _vanishing_filter(float(j), jCut, jMax) if c.Nj > 2 else 1.0
            Lr2inv = 0.0 if j == 0 else f2 / (c.g * desc.h0[j])
            damp[i, j] = -prefXY * Qkl * desc.Kh[i] * desc.Kh[i] - prefZ * Qj * Lr2inv
    return damp


def rhs(desc, Ap, Am, A0, t, t0, damping=None):
    """Scheduled RHS: nonlinear advection, then (optionally) adaptive damping
    using max sqrt(u^2+v^2) of the physical velocity."""
    Fp, Fm, F0 = nonlinear_flux(desc, Ap, Am, A0, t, t0)
    if damping is not None:
        fields = inverse_uvweta(desc, Ap, Am, A0, t, t0)
        speed = float(np.max(np.sqrt(fields[0] * fields[0] + fields[1] * fields[1])))
        s = speed * damping
        Fp = Fp + Ap * s
        Fm = Fm + Am * s
        F0 = F0 + A0 * s
    return Fp, Fm, F0


def rk4_step(desc, Ap, Am, A0, t, t0, h, damping=None):
    """WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462)."""
    y = (Ap, Am, A0)
    k = rhs(desc, *y, t, t0, damping)
    wsum = [x.copy() for x in k]
    stage = [y[i] + (0.5 * h) * k[i] for i in range(3)]
    k = rhs(desc, *stage, t + 0.5 * h, t0, damping)
    wsum = [wsum[i] + 2.0 * k[i] for i in range(3)]
    stage = [y[i] + (0.5 * h) * k[i] for i in range(3)]
    k = rhs(desc, *stage, t + 0.5 * h, t0, damping)
    wsum = [wsum[i] + 2.0 * k[i] for i in range(3)]
    stage = [y[i] + h * k[i] for i in range(3)]
    k = rhs(desc, *stage, t + h, t0, damping)
    wsum = [wsum[i] + 1.0 * k[i] for i in range(3)]
    out = [y[i] + (h / 6.0) * wsum[i] for i in range(3)]
    return out[0], out[1], out[2], t + h


def rk4(desc, Ap, Am, A0, t, t0, h, steps, damping=None):
    for _ in range(steps):
        Ap, Am, A0, t = rk4_step(desc, Ap, Am, A0, t, t0, h, damping)
    return Ap, Am, A0, t


def rk4_advance_to_time(desc, Ap, Am, A0, t, t0, final, h, damping=None):
    """WVFixedStepRK4::advanceToTime (WVRungeKutta.cpp:464-480) with retained
    dense output: steps of min(h, final - t) until final.  Returns (Ap, Am, A0,
    final, dense) where dense = (t_i, t_f, y_i, y_f, k1, k4) of the last step:
    the state before and after it, its first stage derivative and its fourth
    (f at t_i + h of y_i + h k3)."""
    y = [Ap, Am, A0]
    dense = None
    while t < final:
        step = min(h, final - t)
        if not step > 0.0:
            break
        k1 = rhs(desc, *y, t, t0, damping)
        wsum = [x.copy() for x in k1]
        st = [y[i] + (0.5 * step) * k1[i] for i in range(3)]
        k = rhs(desc, *st, t + 0.5 * step, t0, damping)
        wsum = [wsum[i] + 2.0 * k[i] for i in range(3)]
        st = [y[i] + (0.5 * step) * k[i] for i in range(3)]
        k = rhs(desc, *st, t + 0.5 * step, t0, damping)
        wsum = [wsum[i] + 2.0 * k[i] for i in range(3)]
        st = [y[i] + step * k[i] for i in range(3)]
        k4 = rhs(desc, *st, t + step, t0, damping)
        wsum = [wsum[i] + 1.0 * k4[i] for i in range(3)]
        y1 = [y[i] + (step / 6.0) * wsum[i] for i in range(3)]
        dense = (t, t + step, y, y1, k1, k4)
        y, t = y1, t + step
    return y[0], y[1], y[2], final, dense


def rk4_dense_output(dense, time):
    """WVFixedStepRK4::evaluateDenseOutput (WVRungeKutta.cpp:482-541): the cubic
    Hermite interpolant through the step's end states with the first and the
    fourth stage derivatives as end slopes."""
    ti, tf, y0, y1, k1, k4 = dense
    h = tf - ti
    theta = 0.0 if h == 0.0 else (time - ti) / h
    theta = max(0.0, min(1.0, theta))
    t2, t3 = theta * theta, theta * theta * theta
    ew = 3 * t2 - 2 * t3
    iw = 1 - ew
    isw = h * (theta - 2 * t2 + t3)
    esw = h * (t3 - t2)
    return [iw * a + ew * b + isw * c + esw * e for a, b, c, e in zip(y0, y1, k1, k4)]


# ---------------------------------------------------------------------------
# Adaptive RK23 (WVAdaptiveRK23, PortableRuntime/src/WVRungeKutta.cpp:554-983)


def rk23_tolerances(desc, abs_scale):
    """Absolute tolerances of the coefficients, (wave, vortex) each (Nkl, Nj):
    wave for A+ and A-, vortex for A0 (WVWaveVortexCoefficientErrorPolicy::create,
    PortableRuntime/src/WVForcingEngine.cpp:79-168).  Radial shells of width
    dK = the widest gap between distinct |K_h| share their width equally among
    their coefficients; tolerance = abs_scale * sqrt(share / energy factor)."""
    c = desc.c
    if not (math.isfinite(abs_scale) and abs_scale > 0.0):
        raise OracleError(1, "Adaptive absolute-tolerance scale must be finite and positive.")
    Kh = [float(v) for v in desc.Kh]
    radii = sorted(set(abs(v) for v in Kh))
    if len(radii) < 2:
        raise OracleError(1, "Adaptive tolerances require at least two distinct horizontal radial wavenumbers.")
    dK = 0.0
    for a, b in zip(radii[:-1], radii[1:]):
        dK = max(dK, b - a)
    centres = []
    centre = 0.0
    while centre <= radii[-1] + 0.5 * dK:
        centres.append(centre)
        centre += dK
    shell = []
    members = [0] * len(centres)
    for kh in Kh:
        for b, ce in enumerate(centres):
            if ce - 0.5 * dK < kh <= ce + 0.5 * dK:
                shell.append(b)
                members[b] += 1
                break
        else:
            raise OracleError(1, "A horizontal mode was not assigned to an adaptive radial tolerance bin.")
    wave = np.ones((len(Kh), c.Nj))
    vortex = np.ones((len(Kh), c.Nj))
    f2 = desc.f * desc.f
    N02 = c.N0 * c.N0
    for i, kh in enumerate(Kh):
        ce = centres[shell[i]]
        share = (ce + 0.5 * dK - max(ce - 0.5 * dK, 0.0)) / members[shell[i]]
        for j in range(c.Nj):
            m = float(desc.m[j])
            we = 0.0
            if kh == 0.0:
                we = c.Lz if j == 0 else (N02 / (c.g * m * m) if c.isHydrostatic else (N02 - f2) / (c.g * m * m))
            elif j > 0:
                we = 2.0 * (N02 / (c.g * m * m) if c.isHydrostatic else (N02 - f2) / (c.g * (m * m + kh * kh)))
            ve = 0.0
            if kh > 0.0:
                ld2 = 0.0 if j == 0 else f2 / (c.g * float(desc.h0[j]))
                ve = float(desc.h0[j]) / (kh * kh + ld2)
            elif j > 0:
                ve = c.g / 2.0
            if we > 0.0 and math.isfinite(we):
                wave[i, j] = abs_scale * math.sqrt(share / we)
            if ve > 0.0 and math.isfinite(ve):
                vortex[i, j] = abs_scale * math.sqrt(share / ve)
    return wave, vortex


def rk23_tolerance_hash(components):
    """toleranceHash / toleranceComponentHashes (WVRungeKutta.cpp:26-37,602-613):
    FNV-1a over the tolerances rounded to 32 significand bits."""
    mask = (1 << 64) - 1
    total = 1469598103934665603
    per = []
    for comp in components:
        bits = np.ascontiguousarray(comp, dtype=np.float64).reshape(-1).view(np.uint64)
        hc = 1469598103934665603
        for b in bits.tolist():
            v = (b + 0x80000) & ~0xFFFFF & mask
            total = ((total ^ v) * 1099511628211) & mask
            hc = ((hc ^ v) * 1099511628211) & mask
        per.append(hc)
    return total, per


RK23_DEFAULTS = dict(rtol=1e-3, atol_scale=1e-6, safety=0.8, floor=0.5, max_factor=5.0, max_step=math.inf,
                     max_diagnostics=512)


class RK23:
    """WVAdaptiveRK23 over a right-hand side f(y, t) -> list of arrays, y a list
    of complex arrays with absolute tolerances atol (same shapes): Bogacki-
    Shampine 3(2) stages, first-same-as-last reuse, the "matlab-ode23-v1"
    controller (WVRungeKutta.cpp:660-890), advanceToTime (:892-912) and the
    cubic dense output (:914-981).  State constraints of the constant-
    stratification system (forcing-amplitude restoration) are empty for the
    advection and damping schedules and so are omitted."""

    B = (2.0 / 9.0 - 7.0 / 24.0, 1.0 / 3.0 - 0.25, 4.0 / 9.0 - 1.0 / 3.0)

    def __init__(self, f, atol, **options):
        self.f = f
        self.atol = atol
        self.o = {**RK23_DEFAULTS, **options}
        self.k1 = self.k4 = None
        self.fsal = False
        self.next_step = 0.0
        self.accepted = None
        self.evaluations = 0
        self.accepted_steps = 0
        self.rejected_steps = 0
        self.fsal_reuses = 0
        self.diagnostics = []

    @staticmethod
    def time_tolerance(a, b):
        return 8.0 * np.finfo(float).eps * max(1.0, abs(a), abs(b))

    def _eval(self, y, t):
        self.evaluations += 1
        return [np.asarray(v) for v in self.f(y, t)]

    def step(self, y, t, proposed):
        """Returns (y_next, t_next) of one accepted step."""
        o = self.o
        if not (proposed > 0.0 and math.isfinite(proposed)):
            raise OracleError(1, "RK23 step size must be finite and positive.")
        self.accepted = None
        h = min(proposed, o["max_step"])
        have_first = reused = False
        if self.fsal:
            self.k1 = self.k4
            have_first = reused = True
            self.fsal = False
            self.fsal_reuses += 1
        rejected = evals = 0
        while True:
            if not math.isfinite(h) or not (t + h > t):
                raise OracleError(9, "RK23 cannot advance time with the proposed step.")
            if not have_first:
                self.k1 = self._eval(y, t)
                evals += 1
                have_first = True
            k1 = self.k1
            stage = [y[c] + (0.5 * h) * k1[c] for c in range(len(y))]
            k2 = self._eval(stage, t + 0.5 * h)
            stage = [y[c] + (0.75 * h) * k2[c] for c in range(len(y))]
            k3 = self._eval(stage, t + 0.75 * h)
            s1, s2, s3 = h * (2.0 / 9.0), h * (1.0 / 3.0), h * (4.0 / 9.0)
            cand = [((y[c] + s1 * k1[c]) + s2 * k2[c]) + s3 * k3[c] for c in range(len(y))]
            k4 = self._eval(cand, t + h)
            evals += 3
            b1, b2, b3 = self.B
            error = 0.0
            for c in range(len(y)):
                e = h * (((b1 * k1[c] + b2 * k2[c]) + b3 * k3[c]) - 0.125 * k4[c])
                with np.errstate(divide="ignore", invalid="ignore"):
                    scale = np.maximum(self.atol[c], o["rtol"] * np.maximum(np.abs(y[c]), np.abs(cand[c])))
                    ratio = np.abs(e) / scale
                if not np.all(np.isfinite(ratio)):
                    error = math.inf
                    break
                error = max(error, float(np.max(ratio)) if ratio.size else 0.0)
            ok = math.isfinite(error) and error <= 1.0
            factor = 1.0
            if ok:
                if rejected == 0:
                    temp = 1.25 * np.cbrt(error)
                    factor = 1.0 / temp if temp > 0.2 else o["max_factor"]
            elif rejected == 0:
                factor = max(o["floor"], o["safety"] * error ** (-1.0 / 3.0))
            else:
                factor = o["floor"]
            self.next_step = min(o["max_step"], h * factor)
            self.normalized_error = error
            if ok:
                self.k2, self.k3, self.k4 = k2, k3, k4
                self.accepted = (t, t + h, cand)
                self.accepted_steps += 1
                self.fsal = True
                if len(self.diagnostics) < o["max_diagnostics"]:
                    self.diagnostics.append((t, h, error, self.next_step, rejected, evals, reused))
                return cand, t + h
            rejected += 1
            self.rejected_steps += 1
            h = self.next_step
            if not (h > 0.0) or t + h == t:
                raise OracleError(9, "RK23 step size underflowed after rejection.")

    def advance_to_time(self, y, t, final, h):
        if final < t or not math.isfinite(final):
            raise OracleError(1, "RK23 cannot advance backward or to a nonfinite time.")
        while t < final:
            remaining = final - t
            if remaining <= self.time_tolerance(t, final):
                break
            y, t = self.step(y, t, min(h, remaining))
            h = self.next_step
        return y, final

    def dense_output(self, time):
        if self.accepted is None:
            raise OracleError(10, "RK23 dense output is unavailable.")
        ti, tf, end = self.accepted
        h = tf - ti
        tol = self.time_tolerance(ti, tf)
        if time < ti - tol or time > tf + tol:
            raise OracleError(1, "Dense-output time is outside the accepted interval.")
        theta = 0.0 if h == 0 else (time - ti) / h
        if abs(time - ti) <= tol:
            theta = 0.0
        if abs(time - tf) <= tol:
            theta = 1.0
        theta = max(0.0, min(1.0, theta))
        t2 = theta * theta
        t3 = t2 * theta
        w = (theta - (4.0 / 3.0) * t2 + (5.0 / 9.0) * t3 - 2.0 / 9.0, t2 - (2.0 / 3.0) * t3 - 1.0 / 3.0,
             (4.0 / 3.0) * t2 - (8.0 / 9.0) * t3 - 4.0 / 9.0, -t2 + t3)
        ks = (self.k1, self.k2, self.k3, self.k4)
        out = []
        for c in range(len(end)):
            v = end[c].copy()
            for d in range(4):
                v = v + (h * w[d]) * ks[d][c]
            out.append(v)
        return out


def _wrapped(c, L):
    """wrapped() of WVFieldEvaluationService.cpp:107-114."""
    v = math.fmod(c, L)
    if v < 0.0:
        v += L
    if v >= L:
        v = 0.0
    return v


def particle_velocity_linear(desc, fields, x, y, z, nch):
    """Linear branch of evaluateMovingImpl (WVFieldEvaluationService.cpp:1951-1985):
    trilinear interpolation of fields (3, Nz, Ny, Nx) at unwrapped (x, y) and z,
    periodic in x and y, zero outside -Lz <= z <= 0.  Returns (nch, n)."""
    c = desc.c
    dx, dy, dz = c.Lx / c.Nx, c.Ly / c.Ny, c.Lz / (c.Nz - 1)
    out = np.zeros((nch, len(x)))
    for p in range(len(x)):
        xx, yy, zz = _wrapped(float(x[p]), c.Lx), _wrapped(float(y[p]), c.Ly), float(z[p])
        if not (-c.Lz <= zz <= 0.0):
            continue
        x0 = min(int(math.floor(xx / dx)), c.Nx - 1)
        y0 = min(int(math.floor(yy / dy)), c.Ny - 1)
        nz = (zz + c.Lz) / dz
        z0 = min(int(max(0.0, math.floor(nz))), c.Nz - 2)
        wx1 = (xx - x0 * dx) / dx
        wy1 = (yy - y0 * dy) / dy
        wz1 = min(max(nz - z0, 0.0), 1.0)
        xi, yi = (x0, (x0 + 1) % c.Nx), (y0, (y0 + 1) % c.Ny)
        wx, wy, wz = (1.0 - wx1, wx1), (1.0 - wy1, wy1), (1.0 - wz1, wz1)
        for ch in range(nch):
            v = 0.0
            for iz in range(2):
                for iy in range(2):
                    for ix in range(2):
                        v += float(fields[ch][z0 + iz, yi[iy], xi[ix]]) * wx[ix] * wy[iy] * wz[iz]
            out[ch, p] = v
    return out


def spline_weights(n, origin, spacing, query, shift=0):
    """SplineSystem::weightsInto (WVFieldEvaluationService.cpp:116-230): weights
    over all n points of the not-a-knot cubic spline through uniform samples,
    linear for n = 2 and quadratic for n = 3; `shift` rotates the result back
    (restoreOriginalOrdering)."""
    normalized = (query - origin) / spacing
    if n == 2:
        shifted = np.array([1.0 - normalized, normalized])
    elif n == 3:
        shifted = np.array([(normalized - 1.0) * (normalized - 2.0) / 2.0, -normalized * (normalized - 2.0),
                            normalized * (normalized - 1.0) / 2.0])
    else:
        interval = 0 if normalized <= 0.0 else int(math.floor(normalized))
        interval = min(interval, n - 2)
        fraction = min(max(normalized - interval, 0.0), 1.0)
        first, second = 1.0 - fraction, fraction
        A = np.zeros((n, n))
        A[0, :3] = (-1.0, 2.0, -1.0)
        for r in range(1, n - 1):
            A[r, r - 1:r + 2] = (1.0, 4.0, 1.0)
        A[n - 1, n - 3:] = (-1.0, 2.0, -1.0)
        rhs = np.zeros(n)
        rhs[interval] = (first ** 3 - first) * spacing * spacing / 6.0
        rhs[interval + 1] = (second ** 3 - second) * spacing * spacing / 6.0
        cvec = np.linalg.solve(A.T, rhs)
        shifted = np.zeros(n)
        shifted[interval] += first
        shifted[interval + 1] += second
        scale = 6.0 / (spacing * spacing)
        for r in range(1, n - 1):
            shifted[r - 1] += scale * cvec[r]
            shifted[r] -= 2.0 * scale * cvec[r]
            shifted[r + 1] += scale * cvec[r]
    out = np.zeros(n)
    for s in range(n):
        out[(s + n - shift % n) % n] += shifted[s]
    return out


def particle_velocity_spline(desc, fields, x, y, z, nch):
    """Spline branch of evaluateMovingImpl (WVFieldEvaluationService.cpp:1986-2016):
    x and y move four cells away from the periodic seam when within three
    cells of it, weights over the whole grid, value = sum f wx wy wz."""
    c = desc.c
    dx, dy, dz = c.Lx / c.Nx, c.Ly / c.Ny, c.Lz / (c.Nz - 1)
    out = np.zeros((nch, len(x)))
    for p in range(len(x)):
        xx, yy, zz = _wrapped(float(x[p]), c.Lx), _wrapped(float(y[p]), c.Ly), float(z[p])
        if not (-c.Lz <= zz <= 0.0):
            continue
        xl = min(int(math.floor(xx / dx)), c.Nx - 1)
        yl = min(int(math.floor(yy / dy)), c.Ny - 1)
        xb = xl < 3 or xl > c.Nx - 4
        yb = yl < 3 or yl > c.Ny - 4
        xq = _wrapped(xx + 4.0 * dx, c.Lx) if xb else xx
        yq = _wrapped(yy + 4.0 * dy, c.Ly) if yb else yy
        if not (xq <= (c.Nx - 1) * dx and yq <= (c.Ny - 1) * dy):
            continue
        wx = spline_weights(c.Nx, 0.0, dx, xq, 4 if xb else 0)
        wy = spline_weights(c.Ny, 0.0, dy, yq, 4 if yb else 0)
        wz = spline_weights(c.Nz, -c.Lz, dz, zz, 0)
        for ch in range(nch):
            out[ch, p] = float(np.einsum("zyx,x,y,z->", fields[ch], wx, wy, wz))
    return out


@dataclass
class ParticleGroup:
    """A WVLagrangianParticles observer: x, y (and z unless xy_only) state
    blocks; z holds the fixed depths of an xy-only group."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    xy_only: bool = False
    spline: bool = False
    horizontal_tolerance: float = 1e-5
    vertical_tolerance: float = 1e-6


@dataclass
class Tracer:
    """A three-dimensional WVTracer observer."""

    antialias: bool = True
    tolerance: float = 1e-8


def system_state(desc, Ap, Am, A0, groups, tracers):
    """Initial integration state [Ap, Am, A0, blocks...] with the particle
    positions of each group (x, y[, z]) and one (Nz, Ny, Nx) field per tracer."""
    y = [Ap, Am, A0]
    for g in groups:
        y += [np.array(g.x, float), np.array(g.y, float)] + ([] if g.xy_only else [np.array(g.z, float)])
    for tr, field in tracers:
        y.append(np.array(field, float))
    return y


def system_rhs(desc, y, t, t0, groups, tracers, damping=None):
    """WVConstantStratificationIntegrationSystem::evaluateRightHandSide
    (PortableRuntime/src/WVConstantStratificationIntegrationSystem.cpp:295-400):
    the scheduled flux, then each particle group's velocity at its positions and
    each tracer's F-grid advection, all from the advection fields (u, v, w) of
    the state.  `tracers` is a list of Tracer (their fields are in y)."""
    Ap, Am, A0 = y[0], y[1], y[2]
    out = list(rhs(desc, Ap, Am, A0, t, t0, damping))
    adv = velocity_fields(desc, Ap, Am, A0, t, t0)
    i = 3
    for g in groups:
        px, py = y[i], y[i + 1]
        pz = np.asarray(g.z, float) if g.xy_only else y[i + 2]
        nch = 2 if g.xy_only else 3
        vel = (particle_velocity_spline if g.spline else particle_velocity_linear)(desc, adv, px, py, pz, nch)
        out += [vel[c] for c in range(nch)]
        i += nch
    for tr in tracers:
        out.append(advect_fgrid_scalar(desc, y[i], adv, tr.antialias))
        i += 1
    return out


def system_rk4(desc, y, t, t0, h, steps, groups, tracers, damping=None):
    """WVFixedStepRK4::step over the extended state (WVRungeKutta.cpp:335-462)."""
    f = lambda v, tt: system_rhs(desc, v, tt, t0, groups, tracers, damping)
    for _ in range(steps):
        k = f(y, t)
        wsum = [a.copy() for a in k]
        st = [a + (0.5 * h) * b for a, b in zip(y, k)]
        k = f(st, t + 0.5 * h)
        wsum = [a + 2.0 * b for a, b in zip(wsum, k)]
        st = [a + (0.5 * h) * b for a, b in zip(y, k)]
        k = f(st, t + 0.5 * h)
        wsum = [a + 2.0 * b for a, b in zip(wsum, k)]
        st = [a + h * b for a, b in zip(y, k)]
        k = f(st, t + h)
        wsum = [a + 1.0 * b for a, b in zip(wsum, k)]
        y = [a + (h / 6.0) * b for a, b in zip(y, wsum)]
        t = t + h
    return y, t


def system_tolerances(desc, abs_scale, groups, tracers):
    """Absolute tolerances of every state component (UnifiedErrorPolicy,
    WVConstantStratificationIntegrationSystem.cpp:47-86): the coefficient
    policy for A+, A-, A0, each block's uniform tolerance after them."""
    wave, vortex = rk23_tolerances(desc, abs_scale)
    tol = [wave, wave, vortex]
    for g in groups:
        n = len(g.x)
        tol += [np.full(n, g.horizontal_tolerance)] * 2
        if not g.xy_only:
            tol.append(np.full(n, g.vertical_tolerance))
    c = desc.c
    for tr in tracers:
        tol.append(np.full((c.Nz, c.Ny, c.Nx), tr.tolerance))
    return tol


def system_rk23_advance(desc, y, t, t0, final, initial, groups, tracers, damping=None, **options):
    """Adaptive RK23 over the extended state; returns (y, t, integrator)."""
    o = {**RK23_DEFAULTS, **options}
    tol = system_tolerances(desc, o["atol_scale"], groups, tracers)
    rk = RK23(lambda v, tt: system_rhs(desc, v, tt, t0, groups, tracers, damping), tol, **options)
    y, t = rk.advance_to_time(y, t, final, initial)
    return y, t, rk


def rk23_advance(desc, Ap, Am, A0, t, t0, final, initial, damping=None, **options):
    """Adaptive RK23 of the wave-vortex state on the scheduled right-hand side
    from t to final; returns (Ap, Am, A0, t, integrator)."""
    o = {**RK23_DEFAULTS, **options}
    wave, vortex = rk23_tolerances(desc, o["atol_scale"])
    rk = RK23(lambda y, tt: rhs(desc, *y, tt, t0, damping), [wave, wave, vortex], **options)
    y, t = rk.advance_to_time([Ap, Am, A0], t, final, initial)
    return y[0], y[1], y[2], t, rk


# ---------------------------------------------------------------------------
# Energy flux diagnostic (@WVTransform/energyFluxFromNonlinearFlux.m:37-44 with
# total-energy factors of the flow components)


def energy_factors(desc):
    c = desc.c
    Kh = desc.Kh[:, None]
    j = np.arange(c.Nj)[None, :]
    hpm = desc.hpm
    Apm = np.where((Kh > 0) & (j > 0), 2.0 * hpm, 0.0)
    Apm = np.where((Kh == 0) & (j > 0), hpm, Apm)
    Apm = np.where((Kh == 0) & (j == 0), c.Lz, Apm)
    f2 = desc.f * desc.f
    K2 = Kh * Kh
    with np.errstate(divide="ignore", invalid="ignore"):
        Lr2inv = np.where(j == 0, 0.0, f2 / (c.g * desc.h0[None, :]))
        geo_j = (K2 * desc.h0[None, :] + f2 / c.g) / ((K2 + Lr2inv) ** 2)
        geo_0 = c.Lz / K2
    A0f = np.where((Kh > 0) & (j > 0), geo_j, 0.0)
    A0f = np.where((Kh > 0) & (j == 0), geo_0, A0f)
    A0f = np.where((Kh == 0) & (j > 0), c.g / 2.0, A0f)
    return Apm, A0f


def energy_flux(desc, Ap, Am, A0, Fp, Fm, F0):
    Apm_f, A0_f = energy_factors(desc)
    Ep = 2.0 * Apm_f * np.real(Fp * np.conj(Ap))
    Em = 2.0 * Apm_f * np.real(Fm * np.conj(Am))
    E0 = 2.0 * A0_f * np.real(F0 * np.conj(A0))
    return Ep, Em, E0


# ---------------------------------------------------------------------------
# Synthetic states


def random_state(desc, seed, scale=1e-3):
    """Seeded arbitrary complex coefficients (not necessarily representable)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = (desc.Nkl, desc.c.Nj)
    out = []
    for _ in range(3):
        out.append(scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
    return tuple(out)


def spectrum_state(desc, seed, urms=0.1, t0=0.0):
    """Seeded state with uniform random phases and Gaussian amplitudes shaped by
    the isotropic spectrum (Kh^2 + (j*pi/Lz)^2)^(-3/4) in amplitude (energy
    ~ (Kh^2+m^2)^(-3/2)), made representable by one inverse->forward round trip
    and scaled to the requested rms velocity."""
    c = desc.c
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = (desc.Nkl, c.Nj)
    K2 = desc.Kh[:, None] ** 2 + (np.arange(c.Nj)[None, :] * PI / c.Lz) ** 2
    with np.errstate(divide="ignore"):
        env = np.where(K2 > 0, K2 ** (-0.75), 0.0)
    comps = []
    for _ in range(3):
        amp = rng.standard_normal(shape) * env
        ph = rng.uniform(0.0, 2.0 * PI, shape)
        comps.append(amp * np.exp(1j * ph))
    Ap, Am, A0 = comps
    fields = inverse_uvweta(desc, Ap, Am, A0, t0, t0)
    Ap, Am, A0 = forward(desc, fields[[0, 1, 3]] if c.isHydrostatic else fields, t0, t0)
    fields = inverse_uvweta(desc, Ap, Am, A0, t0, t0)
    rms = math.sqrt(float(np.mean(fields[0] ** 2 + fields[1] ** 2 + fields[2] ** 2)))
    s = urms / rms if rms > 0 else 1.0
    return Ap * s, Am * s, A0 * s


def cfl_time_step(desc, Ap, Am, A0, t0=0.0, cfl=0.5):
    """Fixed-step dt per WVModelFixedTimeStepMethods.timeStepForCFL
    (Integrators/WVModelFixedTimeStepMethods.m:50-95): cfl times the minimum of
    dx_eff/max|u_h|, (3/2)dz/max|w| (levels above the bottom) and the period
    of the fastest resolved wave (j >= 1)."""
    c = desc.c
    fields = inverse_uvweta(desc, Ap, Am, A0, t0, t0)
    U = float(np.max(np.sqrt(fields[0] ** 2 + fields[1] ** 2)))
    dx = PI / float(np.max(np.maximum(np.abs(desc.k), np.abs(desc.l))))
    dz = c.Lz / (c.Nz - 1)
    Wm = float(np.max(np.abs(fields[2][1:])))
    advective = cfl * dx / U if U > 0 else float("inf")
    if Wm > 0:
        advective = min(advective, cfl * (1.5 * dz) / Wm)
    omax = float(np.max(np.abs(desc.arrays["omega"][:, 1:]))) if c.Nj > 1 else 0.0
    oscillatory = cfl * 2.0 * PI / omax if omax > 0 else float("inf")
    return min(advective, oscillatory)


# ---------------------------------------------------------------------------
# Second summation order for the vertical transforms (noise-floor estimate).
# Exact dense DCT-I / DST-I matrices with integer argument reduction.  Two
# valid FP64 evaluations of the same flux differ by the computation's own
# rounding noise; tests use that difference as the floor of attainable parity.

import contextlib


def _cospi(a, b):
    r = np.mod(a, 2 * b)
    return np.cos(PI * r / b)


def _sinpi(a, b):
    r = np.mod(a, 2 * b)
    out = np.sin(PI * r / b)
    out[(r == 0) | (r == b)] = 0.0
    return out


def _dct1_dense(x, axis):
    x = np.moveaxis(x, axis, -1)
    n = x.shape[-1]
    k = np.arange(n)
    C = 2.0 * _cospi(np.outer(k, k), n - 1)
    C[:, 0] = 1.0
    C[:, -1] = (-1.0) ** k
    return np.moveaxis(x @ C.T, -1, axis)


def _dst1_dense(x, axis):
    x = np.moveaxis(x, axis, -1)
    n = x.shape[-1]
    k = np.arange(1, n + 1)
    S = 2.0 * _sinpi(np.outer(k, k), n + 1)
    return np.moveaxis(x @ S.T, -1, axis)


@contextlib.contextmanager
def dense_vertical():
    """Evaluate the vertical transforms as exact dense matrix products instead
    of FFT-based DCT-I/DST-I (same mathematics, different rounding)."""
    global _dct1, _dst1
    saved = (_dct1, _dst1)
    _dct1, _dst1 = _dct1_dense, _dst1_dense
    try:
        yield
    finally:
        _dct1, _dst1 = saved


def noise_floor(fn, *args, **kwargs):
    """(result, floor): result of fn with FFT-based vertical transforms and the
    per-output relative difference (max|diff|/max|ref|) to the dense ordering."""
    ref = fn(*args, **kwargs)
    with dense_vertical():
        alt = fn(*args, **kwargs)
    floors = []
    for a, b in zip(alt, ref):
        den = float(np.max(np.abs(b)))
        floors.append(float(np.max(np.abs(a - b))) / den if den > 0 else 0.0)
    return ref, floors


# ---------------------------------------------------------------------------
# Adjoint (vector-Jacobian products).  No counterpart in the reference; the
# GPU adjoint is checked against this restatement, against central finite
# differences (exact for the quadratic flux up to rounding) and by the
# dot-product test.  Inner product on complex arrays: <a, b> = Re sum conj(a) b.


def _inverse_matrices(desc):
    """(Nz, Nj) real matrices of the inverse vertical transforms with the x0.5
    coefficient-production scaling: value channels (cos, sin) and the
    z-derivative channels (-m sin for cosine fields, +m cos for sine fields)."""
    c = desc.c
    z = np.arange(c.Nz)[:, None]
    j = np.arange(c.Nj)[None, :]
    L = c.Nz - 1
    ccos = np.where(j == 0, 0.5, _cospi(j * z, L))
    csin = np.where((j >= 1) & (z >= 1) & (z <= c.Nz - 2), _sinpi(j * z, L), 0.0)
    m = desc.m[None, :]
    return ccos, csin, -m * csin, m * ccos


def _forward_matrices(desc):
    """(Nj, Nz) forward vertical matrices (DCT-I / DST-I + normalization) times
    the horizontal scale 1/(Nx Ny)."""
    c = desc.c
    n = np.arange(c.Nz)[None, :]
    j = np.arange(c.Nj)[:, None]
    L = c.Nz - 1
    fc = np.where(n == 0, 1.0, np.where(n == c.Nz - 1, (-1.0) ** j, 2.0 * _cospi(j * n, L)))
    fc = np.where(j == c.Nz - 1, 0.5 * fc, fc) / L
    fs = np.where((j >= 1) & (n >= 1) & (n <= c.Nz - 2), 2.0 * _sinpi(j * n, L), 0.0) / L
    hs = 1.0 / float(c.Nx * c.Ny)
    return fc * hs, fs * hs


def _rows_to_columns_adjoint(desc, half_rows):
    """Adjoint of _columns_to_half for one channel: (rows, Nz) -> (Nkl, Nz) in
    the WV frame (completion rows folded back conjugated, self-conjugate rows
    real, conjugated storage undone)."""
    h = half_rows.copy()
    if len(desc.completionRows):
        np.add.at(h, desc.completionSources, np.conj(h[desc.completionRows]))
    if len(desc.selfConjugateRows):
        h[desc.selfConjugateRows] = h[desc.selfConjugateRows].real
    v = h[desc.storageRow]
    return np.where(desc.conjugated[:, None], np.conj(v), v)


def _c2r_adjoint(desc, fields):
    """Adjoint of the unnormalized c2r (FFTW semantics): fields (ch, Nz, Ny, Nx)
    -> half rows (ch, rows, Nz); interior kx carry weight 2."""
    h = _spatial_to_half_rows(desc, fields)
    c = desc.c
    kx = np.arange(desc.NxHalf)
    w = np.where((kx == 0) | (2 * kx == c.Nx), 1.0, 2.0)
    wr = np.tile(w, c.Ny)  # row = kx + NxHalf*ky
    return h * wr[None, :, None]


def _r2c_adjoint(desc, half_rows):
    """Adjoint of the unnormalized r2c: half rows (ch, rows, Nz) -> fields
    Re sum_{kx<=Nx/2} H e^{+i...} (interior kx at weight 1/2 under c2r)."""
    c = desc.c
    kx = np.arange(desc.NxHalf)
    w = np.where((kx == 0) | (2 * kx == c.Nx), 1.0, 0.5)
    wr = np.tile(w, c.Ny)
    return _half_rows_to_spatial(desc, half_rows * wr[None, :, None])


def flux_vjp(desc, Ap, Am, A0, t, t0, Fpb, Fmb, F0b):
    """Adjoint of nonlinear_flux: returns (Apb, Amb, A0b) with
    <(Fpb, Fmb, F0b), dF> = <(Apb, Amb, A0b), dA> for every perturbation dA."""
    c = desc.c
    a = desc.arrays
    p = phase(desc, t, t0)
    targets = (0, 1, 3) if c.isHydrostatic else (0, 1, 2, 3)
    ccos, csin, csinm, ccosm = _inverse_matrices(desc)
    fcos, fsin = _forward_matrices(desc)
    kC = desc.k[:, None]
    lC = desc.l[:, None]
    vort, buoyF, na0, apmn = a["A0FromVorticity"], a["A0FromBuoyancy"], a["NA0"], a["ApmN"]
    cpb = Fpb * p
    cmb = Fmb * np.conj(p)
    a0b = F0b
    # recomputed forward fields
    U, V, W = velocity_fields(desc, Ap, Am, A0, t, t0)
    fb = {f: np.zeros_like(Ap) for f in range(4)}  # field-value adjoints u, v, w, eta (WV frame, j space)
    grad_U = np.zeros_like(U)
    grad_V = np.zeros_like(V)
    grad_W = np.zeros_like(W)
    for q in targets:
        # projection adjoint -> value bar (Nkl, Nj)
        wave_b = cpb + cmb
        buoy_b = cpb - cmb
        bv_b = buoy_b * apmn
        A0c_b = a0b - na0 * bv_b
        vb = np.zeros_like(Ap)
        if q == 3:
            vb = vb + bv_b
        if q == 0:
            vb = vb + (1j * lC) * vort * A0c_b
        elif q == 1:
            vb = vb + (-1j * kC) * vort * A0c_b
        elif q == 3:
            vb = vb + buoyF * A0c_b
        if c.isHydrostatic:
            if q == 0:
                vb = vb + (-1j * kC) * np.conj(a["ApmD"]) * wave_b
            elif q == 1:
                vb = vb + (-1j * lC) * np.conj(a["ApmD"]) * wave_b
        else:
            if q == 0:
                vb = vb + (desc.cosAlpha[:, None] * a["ApmDScaled"]) * wave_b
            elif q == 1:
                vb = vb + (desc.sinAlpha[:, None] * a["ApmDScaled"]) * wave_b
            elif q == 2:
                sc = (desc.Kh[:, None] / 2.0) * desc.apmWProjectionPrefactor[None, :]
                vb = vb + (-1j * sc) * wave_b
        # inertial mode (WV index 0): contributions overridden
        sc0 = desc.inertialScale
        tot = cpb[0] + np.conj(cmb[0])
        v0 = np.zeros(c.Nj, np.complex128)
        if q == 0:
            v0 = sc0 * tot
        elif q == 1:
            v0 = (1j * sc0) * tot
        if q == 3:
            v0 = v0 + buoyF[0] * a0b[0]
        vb[0] = v0
        # forward vertical adjoint: (Nkl, Nj) -> (Nkl, Nz)
        F = fcos if q < 2 else fsin
        col_b = vb @ F
        # scatter to stored rows (conjugated storage), then adjoint of r2c -> S bar
        half = np.zeros((1, c.Ny * desc.NxHalf, c.Nz), np.complex128)
        half[0, desc.storageRow, :] = np.where(desc.conjugated[:, None], np.conj(col_b), col_b)
        Sb = _r2c_adjoint(desc, half)[0]
        # products adjoint with the recomputed forward derivative fields
        dx, dy, dz = derivative_fields(desc, Ap, Am, A0, t, t0, q)
        grad_U -= Sb * dx
        grad_V -= Sb * dy
        grad_W -= Sb * dz
        gx, gy, gz = -Sb * U, -Sb * V, -Sb * W
        hb = _c2r_adjoint(desc, np.stack([gx, gy, gz]))
        cx_ = _rows_to_columns_adjoint(desc, hb[0])
        cy_ = _rows_to_columns_adjoint(desc, hb[1])
        cz_ = _rows_to_columns_adjoint(desc, hb[2])
        Cv = ccos if q < 2 else csin
        Cz = csinm if q < 2 else ccosm
        fb[q] = fb[q] + (-1j * kC) * (cx_ @ Cv) + (-1j * lC) * (cy_ @ Cv) + cz_ @ Cz
    # advecting velocity adjoints
    hb = _c2r_adjoint(desc, np.stack([grad_U, grad_V, grad_W]))
    fb[0] = fb[0] + _rows_to_columns_adjoint(desc, hb[0]) @ ccos
    fb[1] = fb[1] + _rows_to_columns_adjoint(desc, hb[1]) @ ccos
    fb[2] = fb[2] + _rows_to_columns_adjoint(desc, hb[2]) @ csin
    return _assembly_adjoint(desc, fb[0], fb[1], fb[2], fb[3], p)


def _assembly_adjoint(desc, ub, vb, wb, nb, p):
    """Adjoint of _field_values (coefficientValueForField on evolved coefficients)."""
    a = desc.arrays
    Apeb = np.conj(a["UAp"]) * ub + np.conj(a["VAp"]) * vb + np.conj(a["WAp"]) * wb + a["NAp"] * nb
    Ameb = a["UAp"] * ub + a["VAp"] * vb + np.conj(a["WAp"]) * wb - a["NAp"] * nb
    A0b = np.conj(a["UA0"]) * ub + np.conj(a["VA0"]) * vb + a["NA0"] * nb
    return Apeb * np.conj(p), Ameb * p, A0b


def inverse_vjp(desc, t, t0, fields_bar):
    """Adjoint of inverse_uvweta: fields_bar (4, Nz, Ny, Nx) -> (Apb, Amb, A0b)."""
    ccos, csin, _, _ = _inverse_matrices(desc)
    p = phase(desc, t, t0)
    hb = _c2r_adjoint(desc, fields_bar)
    ub = _rows_to_columns_adjoint(desc, hb[0]) @ ccos
    vb = _rows_to_columns_adjoint(desc, hb[1]) @ ccos
    wb = _rows_to_columns_adjoint(desc, hb[2]) @ csin
    nb = _rows_to_columns_adjoint(desc, hb[3]) @ csin
    return _assembly_adjoint(desc, ub, vb, wb, nb, p)


def rk4_step_vjp(desc, Ap, Am, A0, t, t0, h, yb):
    """Adjoint of rk4_step (no damping): given the cotangent of y_{n+1},
    returns the cotangent of y_n.  Stage states are recomputed from y_n."""
    y = (Ap, Am, A0)
    k1 = nonlinear_flux(desc, *y, t, t0)
    s2 = [y[i] + (0.5 * h) * k1[i] for i in range(3)]
    k2 = nonlinear_flux(desc, *s2, t + 0.5 * h, t0)
    s3 = [y[i] + (0.5 * h) * k2[i] for i in range(3)]
    k3 = nonlinear_flux(desc, *s3, t + 0.5 * h, t0)
    s4 = [y[i] + h * k3[i] for i in range(3)]
    kb4 = [(h / 6.0) * x for x in yb]
    kb3 = [(h / 3.0) * x for x in yb]
    kb2 = [(h / 3.0) * x for x in yb]
    kb1 = [(h / 6.0) * x for x in yb]
    out = [x.copy() for x in yb]
    sb = flux_vjp(desc, *s4, t + h, t0, *kb4)
    out = [out[i] + sb[i] for i in range(3)]
    kb3 = [kb3[i] + h * sb[i] for i in range(3)]
    sb = flux_vjp(desc, *s3, t + 0.5 * h, t0, *kb3)
    out = [out[i] + sb[i] for i in range(3)]
    kb2 = [kb2[i] + (0.5 * h) * sb[i] for i in range(3)]
    sb = flux_vjp(desc, *s2, t + 0.5 * h, t0, *kb2)
    out = [out[i] + sb[i] for i in range(3)]
    kb1 = [kb1[i] + (0.5 * h) * sb[i] for i in range(3)]
    sb = flux_vjp(desc, *y, t, t0, *kb1)
    return tuple(out[i] + sb[i] for i in range(3))

"""Test infrastructure only: ctypes binding of oracle/_ref/libwvref.so, the
reference's own CompiledKernel + PortableRuntime subset built by
oracle/ref_build.sh with the C entry layer oracle/ref_shim.cpp.

Used by tests/golden/make_golden.py (fixtures from the exact direct-DFT engine),
by the parity tests at full grids (the O(N log N) oracle FFT engine,
oracle/wv_fft_engine.cpp) and by bench.py's CPU baseline and reference arm.
The GPU library never imports it.

Reference interfaces reached through the shim:
  WVTransformConstantStratificationKernel (CompiledKernel/include/WaveVortexKernel/
    WVTransformConstantStratificationKernel.hpp:47-110)
  WVConstantStratificationIntegrationSystem::evaluateRightHandSide and
    WVFixedStepRK4::step (PortableRuntime/src/WVRungeKutta.cpp:335-462)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libwvref.so")

# Physical constants used for every case unless overridden.
BASE = dict(N0=5.2e-3, rho0=1025.0, g=9.81, planetaryRadius=6.371e6, rotationRate=7.2921e-5)

# FFT providers of the shim (makeEngine in oracle/ref_shim.cpp)
ENGINE_DIRECT = 0
ENGINE_ORACLE_FFT = 1


class Ref:
    """One reference kernel + integration system (+ WVFixedStepRK4) for a case
    dict (Nx, Ny, Nz, Nj, Lx, Ly, Lz, latitude, isHydrostatic, shouldAntialias,
    damping, optional physical constants).  engine: ENGINE_DIRECT (exact,
    O(N^4)) or ENGINE_ORACLE_FFT."""

    def __init__(self, lib, case, engine=ENGINE_DIRECT):
        self.lib = lib
        sizes = (ctypes.c_uint64 * 4)(case["Nx"], case["Ny"], case["Nz"], case["Nj"])
        v = {**BASE, **{k: case[k] for k in case if k in BASE}}
        values = (ctypes.c_double * 9)(case["Lx"], case["Ly"], case["Lz"], v["N0"], v["rho0"], v["g"],
                                       v["planetaryRadius"], v["rotationRate"], case["latitude"])
        flags = (ctypes.c_uint8 * 2)(int(case["isHydrostatic"]), int(case["shouldAntialias"]))
        h = ctypes.c_void_p()
        rc = lib.wvref_create_engine(sizes, values, flags, 1 if case.get("damping") else 0, int(engine), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"wvref_create failed: {rc}")
        self.h = h
        out = (ctypes.c_uint64 * 3)()
        lib.wvref_sizes(h, out)
        self.Nkl, self.NxHalf, self.M = int(out[0]), int(out[1]), int(out[2])
        self.case = case

    def check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.wvref_message(self.h).decode())

    def descriptor(self):
        Nkl, M = self.Nkl, self.M
        kMode = np.zeros(Nkl, np.int64)
        lMode = np.zeros(Nkl, np.int64)
        rows = np.zeros(Nkl, np.uint64)
        conj = np.zeros(Nkl, np.uint8)
        arrs = {n: np.zeros(M) for n in ("omega", "fWaveScale", "A0FromVorticity", "A0FromBuoyancy", "NA0Field",
                                         "ApmNProjection")}
        UAp = np.zeros(M, np.complex128)
        WAp = np.zeros(M, np.complex128)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.lib.wvref_descriptor(self.h, P(kMode), P(lMode), P(arrs["omega"]), P(arrs["fWaveScale"]),
                                  P(arrs["A0FromVorticity"]), P(arrs["A0FromBuoyancy"]), P(arrs["NA0Field"]),
                                  P(arrs["ApmNProjection"]), P(UAp), P(WAp), P(rows), P(conj))
        out = dict(kMode=kMode, lMode=lMode, storageRow=rows.astype(np.int64), conjugated=conj.astype(bool),
                   UApField=UAp, WApField=WAp)
        out.update(arrs)
        return out

    def _c3(self):
        return [np.zeros((self.Nkl, self.case["Nj"]), np.complex128) for _ in range(3)]

    def flux(self, Ap, Am, A0, t, t0, scheduled=False):
        F = self._c3()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        fn = self.lib.wvref_rhs if scheduled else self.lib.wvref_flux
        self.check(fn(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0), P(F[0]), P(F[1]), P(F[2])))
        return F

    def forward(self, fields, t, t0):
        A = self._c3()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_forward(self.h, P(fields), ctypes.c_double(t), ctypes.c_double(t0), P(A[0]), P(A[1]), P(A[2])))
        return A

    def inverse(self, Ap, Am, A0, t, t0):
        c = self.case
        out = np.zeros((4, c["Nz"], c["Ny"], c["Nx"]))
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_inverse(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0), P(out)))
        return out

    def _fields(self, nch):
        c = self.case
        return np.zeros((nch, c["Nz"], c["Ny"], c["Nx"]))

    def flux_with_advection(self, Ap, Am, A0, t, t0):
        F = self._c3()
        adv = self._fields(3)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_flux_with_advection(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0),
                                                      P(F[0]), P(F[1]), P(F[2]), P(adv)))
        return F, adv

    def flux_using_advection(self, Ap, Am, A0, t, t0, adv):
        F = self._c3()
        adv = np.ascontiguousarray(adv)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_flux_using_advection(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0),
                                                       P(F[0]), P(F[1]), P(F[2]), P(adv)))
        return F

    def inverse_uvw(self, Ap, Am, A0, t, t0):
        out = self._fields(3)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_inverse_uvw(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0), P(out)))
        return out

    def field_derivatives(self, Ap, Am, A0, t, t0, field):
        out = self._fields(3)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_field_derivatives(self.h, ctypes.c_double(t), ctypes.c_double(t0), P(Ap), P(Am), P(A0),
                                                    ctypes.c_int(field), P(out)))
        return out

    def advect_scalar(self, scalar, adv, antialias):
        c = self.case
        out = np.zeros((c["Nz"], c["Ny"], c["Nx"]))
        scalar, adv = np.ascontiguousarray(scalar), np.ascontiguousarray(adv)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_advect_scalar(self.h, P(scalar), P(adv), ctypes.c_int(int(antialias)), P(out)))
        return out

    def family_derivatives(self, ffamily, Apm, A0):
        out = self._fields(4)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_family_derivatives(self.h, ctypes.c_int(int(ffamily)), P(Apm), P(A0), P(out)))
        return out

    def rk4(self, Ap, Am, A0, t, t0, dt, steps):
        Ap, Am, A0 = Ap.copy(), Am.copy(), A0.copy()
        tt = ctypes.c_double(t)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.check(self.lib.wvref_rk4(self.h, P(Ap), P(Am), P(A0), ctypes.byref(tt), ctypes.c_double(t0),
                                      ctypes.c_double(dt), ctypes.c_int(steps)))
        return Ap, Am, A0, tt.value

    def rk23(self, Ap, Am, A0, t, t0, final, initial, opts, dense_time=None):
        """opts = (rtol, atol_scale, safety, floor, max_factor, max_step)."""
        Ap, Am, A0 = Ap.copy(), Am.copy(), A0.copy()
        tt = ctypes.c_double(t)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        o = (ctypes.c_double * 6)(*opts)
        cap = 4096
        diag = np.zeros((cap, 7))
        nd = ctypes.c_int()
        counts = (ctypes.c_ulonglong * 4)()
        nxt = ctypes.c_double()
        hashes = (ctypes.c_ulonglong * 4)()
        dense = np.zeros((3,) + Ap.shape, np.complex128) if dense_time is not None else None
        self.check(self.lib.wvref_rk23_advance(
            self.h, o, P(Ap), P(Am), P(A0), ctypes.byref(tt), ctypes.c_double(t0), ctypes.c_double(final),
            ctypes.c_double(initial), P(diag), ctypes.c_int(cap), ctypes.byref(nd), counts, ctypes.byref(nxt), hashes,
            ctypes.c_double(dense_time if dense_time is not None else 0.0), P(dense) if dense is not None else None))
        n = min(nd.value, cap)
        return dict(Ap=Ap, Am=Am, A0=A0, t=tt.value, diag=diag[:n].copy(), counts=np.array(list(counts), np.uint64),
                    next=nxt.value, hashes=np.array(list(hashes), np.uint64), dense=dense)


def load_lib(reference_root=None):
    """Loads libwvref.so, building it first (oracle/ref_build.sh) when absent."""
    if not os.path.exists(LIB):
        cmd = [os.path.join(HERE, "ref_build.sh")] + ([reference_root] if reference_root else [])
        subprocess.check_call(cmd, stdout=subprocess.DEVNULL)
    lib = ctypes.CDLL(LIB)
    lib.wvref_message.restype = ctypes.c_char_p
    lib.wvref_oracle_fft_threads.restype = ctypes.c_uint
    return lib


def available():
    """True when libwvref.so exists or can be built from a staged or checked-out reference."""
    if os.path.exists(LIB):
        return True
    try:
        subprocess.check_call([os.path.join(HERE, "ref_build.sh")], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    except (OSError, subprocess.CalledProcessError):
        return False
    return os.path.exists(LIB)



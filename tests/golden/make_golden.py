"""Generate golden fixtures from the reference's own C++ kernel.

Builds oracle/_ref/libwvref.so from the reference checkout (oracle/ref_build.sh)
and runs the reference CompiledKernel (+ PortableRuntime fixed-step RK4 and
forcing engine) with its exact direct-DFT FFT engine on small seeded cases.
The outputs are written as .npz files next to this script; tests compare the
numpy oracle (oracle/wv_oracle.py) and the GPU path against them.

Usage:  python tests/golden/make_golden.py [REFERENCE_ROOT] [--rk23]
        (REFERENCE_ROOT as oracle/ref_build.sh takes it)
        (--rk23 regenerates only the adaptive RK23 fixture, rk23.npz;
         --system only the integrated-observer fixture, system.npz;
         --rk4-dense only the RK4 advanceToTime / dense-output fixture, rk4_dense.npz)
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from ref_lib import BASE, Ref, load_lib  # noqa: E402

CASES = {
    # 40 km x 40 km x 1 km, 16x16x9, lat 45: single internal wave + adaptive damping
    "wave_16x16x9": dict(Nx=16, Ny=16, Nz=9, Nj=5, Lx=40e3, Ly=40e3, Lz=1000.0, latitude=45.0,
                       isHydrostatic=False, shouldAntialias=True, damping=True, dt=10.0, steps=3),
    # odd grid: 15x13x9 (odd Nx, odd Ny)
    "odd_15x13x9": dict(Nx=15, Ny=13, Nz=9, Nj=5, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0,
                        isHydrostatic=False, shouldAntialias=True, damping=False, dt=20.0, steps=2),
    # the reference's own RK4 test grid (TestWVForcingAndRK4.cpp:66-74), both physics
    "rk_6x5x7": dict(Nx=6, Ny=5, Nz=7, Nj=4, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0, g=9.80665, rho0=1027.0,
                     planetaryRadius=6.3712e6, rotationRate=7.292115e-5,
                     isHydrostatic=False, shouldAntialias=True, damping=False, dt=0.1, steps=2),
    "hydro_8x6x7": dict(Nx=8, Ny=6, Nz=7, Nj=4, Lx=15e3, Ly=12e3, Lz=1300.0, latitude=33.0,
                        isHydrostatic=True, shouldAntialias=True, damping=False, dt=20.0, steps=2),
    # no transform-level antialiasing (the analytic triad test's setting, TestNonlinearFlux.m:68-262)
    "noalias_16x16x9": dict(Nx=16, Ny=16, Nz=9, Nj=5, Lx=4e3, Ly=4e3, Lz=2000.0, latitude=33.0,
                            isHydrostatic=False, shouldAntialias=False, damping=False, dt=20.0, steps=1),
    # rectangular, Nj below the default, hydrostatic with damping
    "hydro_damp_12x10x11": dict(Nx=12, Ny=10, Nz=11, Nj=6, Lx=30e3, Ly=25e3, Lz=2000.0, latitude=-20.0,
                                isHydrostatic=True, shouldAntialias=True, damping=True, dt=15.0, steps=2),
}


def seeded(shape, seed, scale):
    rng = np.random.Generator(np.random.PCG64(seed))
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def main():
    reference_root = sys.argv[1] if len(sys.argv) > 1 else None
    lib = load_lib(reference_root)
    manifest = {}
    for name, case in CASES.items():
        r = Ref(lib, case)
        Nj = case["Nj"]
        shape = (r.Nkl, Nj)
        seed = abs(hash(name)) % 1000  # not used for data; seeds below are fixed per case
        base = sum(ord(ch) for ch in name)
        Ap = seeded(shape, base + 1, 1e-3)
        Am = seeded(shape, base + 2, 1e-3)
        A0 = seeded(shape, base + 3, 1e-3)
        t, t0 = 137.5, -12.25
        desc = r.descriptor()
        Fp, Fm, F0 = r.flux(Ap, Am, A0, t, t0)
        Rp, Rm, R0 = r.flux(Ap, Am, A0, t, t0, scheduled=True)
        nch = 3 if case["isHydrostatic"] else 4
        rng = np.random.Generator(np.random.PCG64(base + 4))
        fields = rng.standard_normal((nch, case["Nz"], case["Ny"], case["Nx"])) * 0.05
        Bp, Bm, B0 = r.forward(fields, t, t0)
        inv = r.inverse(Ap, Am, A0, t, t0)
        # single internal wave state (kMode 1, lMode 0, j 1) for the wave case
        if name.startswith("wave"):
            Sp = np.zeros(shape, np.complex128)
            Sm = np.zeros(shape, np.complex128)
            S0 = np.zeros(shape, np.complex128)
            idx = int(np.nonzero((desc["kMode"] == 1) & (desc["lMode"] == 0))[0][0])
            fws = desc["fWaveScale"].reshape(shape)[idx, 1]
            Sp[idx, 1] = 0.05 / (2.0 * abs(fws))
            rk_in = (Sp, Sm, S0, 0.0, 0.0)
        else:
            rk_in = (Ap, Am, A0, t, t0)
        Kp, Km, K0, tK = r.rk4(rk_in[0], rk_in[1], rk_in[2], rk_in[3], rk_in[4], case["dt"], case["steps"])
        # advection-field entry points, state-field derivatives and F-grid scalar advection
        (Wp, Wm, W0), adv = r.flux_with_advection(Ap, Am, A0, t, t0)
        rng2 = np.random.Generator(np.random.PCG64(base + 5))
        given = rng2.standard_normal((3, case["Nz"], case["Ny"], case["Nx"])) * 0.05
        Up, Um, U0 = r.flux_using_advection(Ap, Am, A0, t, t0, given)
        uvw = r.inverse_uvw(Ap, Am, A0, t, t0)
        fields_deriv = {}
        for q in ((0, 1, 3) if case["isHydrostatic"] else (0, 1, 2, 3)):
            fields_deriv[f"deriv_{q}"] = r.field_derivatives(Ap, Am, A0, t, t0, q)
        scalar = rng2.standard_normal((case["Nz"], case["Ny"], case["Nx"]))
        scal_rhs = r.advect_scalar(scalar, given, False)
        scal_rhs_aa = r.advect_scalar(scalar, given, True)
        Apm = seeded(shape, base + 6, 1e-3)
        fall = r.family_derivatives(True, Apm, A0)
        gall = r.family_derivatives(False, Apm, A0)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            Ap=Ap, Am=Am, A0=A0, t=t, t0=t0,
            Fp=Fp, Fm=Fm, F0=F0, Rp=Rp, Rm=Rm, R0=R0,
            fields=fields, Bp=Bp, Bm=Bm, B0=B0, inverse=inv,
            rk_Ap=rk_in[0], rk_Am=rk_in[1], rk_A0=rk_in[2], rk_t=rk_in[3], rk_t0=rk_in[4],
            rk_dt=case["dt"], rk_steps=case["steps"], Kp=Kp, Km=Km, K0=K0, rk_tout=tK,
            with_Fp=Wp, with_Fm=Wm, with_F0=W0, with_fields=adv, given_fields=given, using_Fp=Up, using_Fm=Um, using_F0=U0,
            uvw=uvw, scalar=scalar, scalar_rhs=scal_rhs, scalar_rhs_aa=scal_rhs_aa, **fields_deriv,
            Apm=Apm, fall=fall, gall=gall,
            **{f"desc_{k}": v for k, v in desc.items()},
        )
        cfg = {k: v for k, v in case.items()}
        cfg.update({k: v for k, v in BASE.items() if k not in case})
        manifest[name] = cfg
        lib.wvref_destroy(r.h)
        print(f"{name}: Nkl={r.Nkl} M={r.M}")
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)
    # 16x16x9 end to end: the single internal wave (kMode=1, lMode=0, j=1, u = 0.05 m/s)
    # under {nonlinear advection, adaptive damping}, 60 RK4 steps of dt = 10 s to t = 600 s
    case = CASES["wave_16x16x9"]
    r = Ref(lib, case)
    shape = (r.Nkl, case["Nj"])
    desc = r.descriptor()
    Sp = np.zeros(shape, np.complex128)
    idx = int(np.nonzero((desc["kMode"] == 1) & (desc["lMode"] == 0))[0][0])
    Sp[idx, 1] = 0.05 / (2.0 * abs(desc["fWaveScale"].reshape(shape)[idx, 1]))
    zero = np.zeros(shape, np.complex128)
    Kp, Km, K0, tK = r.rk4(Sp, zero, zero, 0.0, 0.0, 10.0, 60)
    fields = r.inverse(Kp, Km, K0, tK, 0.0)
    np.savez_compressed(os.path.join(HERE, "wave_16x16x9_t600.npz"), Ap=Sp, Am=zero, A0=zero, dt=10.0, steps=60,
                        Kp=Kp, Km=Km, K0=K0, t=tK, fields=fields)
    lib.wvref_destroy(r.h)
    print(f"wave_16x16x9_t600: t = {tK}")


# Adaptive RK23 runs through the reference integrator (WVAdaptiveRK23):
#   odd:  seeded state, default options, t 100 -> 200 from a 5 s initial step
#   wave: the single internal wave under {advection, damping} to t = 600 s
#   hd:   hydrostatic with damping, every option away from its default
RK23_RUNS = {
    "odd": dict(case="odd_15x13x9", scale=1e-3, t=100.0, t0=0.0, final=200.0, initial=5.0,
                opts=(1e-3, 1e-6, 0.8, 0.5, 5.0, float("inf"))),
    "wave": dict(case="wave_16x16x9", scale=None, t=0.0, t0=0.0, final=600.0, initial=10.0,
               opts=(1e-3, 1e-6, 0.8, 0.5, 5.0, float("inf"))),
    "hd": dict(case="hydro_damp_12x10x11", scale=3e-3, t=50.0, t0=-3.0, final=56.0, initial=40.0,
               opts=(1e-5, 1e-7, 0.9, 0.3, 2.0, 15.0)),
}


def make_rk23(lib):
    out = {}
    for key, run in RK23_RUNS.items():
        case = CASES[run["case"]]
        r = Ref(lib, case)
        shape = (r.Nkl, case["Nj"])
        desc = r.descriptor()
        if run["scale"] is None:
            Ap = np.zeros(shape, np.complex128)
            idx = int(np.nonzero((desc["kMode"] == 1) & (desc["lMode"] == 0))[0][0])
            Ap[idx, 1] = 0.05 / (2.0 * abs(desc["fWaveScale"].reshape(shape)[idx, 1]))
            Am = np.zeros(shape, np.complex128)
            A0 = np.zeros(shape, np.complex128)
        else:
            base = sum(ord(ch) for ch in run["case"]) + 100
            Ap = seeded(shape, base + 1, run["scale"])
            Am = seeded(shape, base + 2, run["scale"])
            A0 = seeded(shape, base + 3, run["scale"])
        # dense output at the midpoint of the last accepted step: run once to learn it
        first = r.rk23(Ap, Am, A0, run["t"], run["t0"], run["final"], run["initial"], run["opts"])
        last = first["diag"][-1]
        mid = last[0] + 0.5 * last[1]
        res = r.rk23(Ap, Am, A0, run["t"], run["t0"], run["final"], run["initial"], run["opts"], dense_time=mid)
        out.update({f"{key}_Ap": Ap, f"{key}_Am": Am, f"{key}_A0": A0, f"{key}_t": run["t"], f"{key}_t0": run["t0"],
                    f"{key}_final": run["final"], f"{key}_initial": run["initial"], f"{key}_opts": np.array(run["opts"]),
                    f"{key}_Kp": res["Ap"], f"{key}_Km": res["Am"], f"{key}_K0": res["A0"], f"{key}_tout": res["t"],
                    f"{key}_diag": res["diag"], f"{key}_counts": res["counts"], f"{key}_next": res["next"],
                    f"{key}_hashes": res["hashes"], f"{key}_dense_time": mid, f"{key}_dense": res["dense"]})
        lib.wvref_destroy(r.h)
        print(f"rk23 {key}: counts {res['counts'].tolist()} t = {res['t']}")
    np.savez_compressed(os.path.join(HERE, "rk23.npz"), **out)


# Integration systems with integrated observers (particle groups and tracers)
# through the reference's WVConstantStratificationIntegrationSystem: one RHS,
# RK4 steps and an adaptive RK23 interval per case.
SYSTEM_RUNS = {
    # the reference's own particle test grid and observers
    # (PortableRuntime/tests/TestWVLagrangianParticles.cpp:86-205)
    "obs": dict(case="rk_6x5x7", schedule=0, coeff="fixture", t=0.25, t0=-0.5, dt=20.0, steps=3,
                groups=[dict(x=[-10.0, 1000.0, 15003.0], y=[20.0, -100.0, 2000.0], z=[-100.0, -300.0, -500.0],
                             xy_only=True, spline=False, tol_h=1e-5, tol_v=1e-6),
                        dict(x=[200.0, 3000.0], y=[400.0, 5000.0], z=[-200.0, -900.0], xy_only=False, spline=True,
                             tol_h=1e-5, tol_v=1e-6)],
                tracers=[dict(antialias=True, tol=1e-8, scale=1.0), dict(antialias=False, tol=1e-8, scale=0.5)],
                rk23=dict(final=60.25, initial=30.0, opts=(1e-6, 1e-8, 0.8, 0.5, 5.0, float("inf")))),
    # hydrostatic with adaptive damping, a linear volume group and a spline xy group
    "hd": dict(case="hydro_damp_12x10x11", schedule=1, coeff="seeded", t=3.0, t0=1.0, dt=5.0, steps=2,
               groups=[dict(x=[1000.0, 17000.0, 29500.0, -400.0], y=[300.0, 12000.0, 24900.0, 5000.0],
                            z=[-100.0, -1000.0, -1999.0, -50.0], xy_only=False, spline=False, tol_h=1e-4, tol_v=1e-5),
                       dict(x=[2600.0, 14100.0, 31000.0], y=[100.0, 9000.0, -2300.0], z=[-300.0, -700.0, -1500.0],
                            xy_only=True, spline=True, tol_h=1e-4, tol_v=1e-5)],
               tracers=[dict(antialias=True, tol=1e-7, scale=2.0)],
               rk23=dict(final=9.0, initial=10.0, opts=(1e-4, 1e-6, 0.8, 0.5, 5.0, 4.0))),
}


def tracer_field(case, scale):
    """initializeTracer of TestWVLagrangianParticles.cpp:271-290 as (Nz, Ny, Nx)."""
    Nx, Ny, Nz = case["Nx"], case["Ny"], case["Nz"]
    z, y, x = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    return scale * (np.sin(2.0 * np.pi * x / Nx) + 0.25 * np.cos(2.0 * np.pi * y / Ny) + 0.1 * np.cos(np.pi * z / (Nz - 1)))


def fixture_coefficients(M):
    """The coefficient pattern of the reference's particle test fixture
    (TestWVLagrangianParticles.cpp:221-231), as three (M,) complex arrays."""
    v = np.arange(1, M + 1, dtype=float)
    return (1e-4 * np.sin(0.17 * v) + 1e-4j * np.cos(0.11 * v), 1e-4 * np.cos(0.13 * v) - 1e-4j * np.sin(0.19 * v),
            1e-4 * np.sin(0.07 * v) + 1e-4j * np.cos(0.23 * v))


def make_system(lib):
    lib.wvref_system_message.restype = ctypes.c_char_p
    lib.wvref_system_extra.restype = ctypes.c_uint64
    out = {}
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for key, run in SYSTEM_RUNS.items():
        case = CASES[run["case"]]
        r = Ref(lib, case)
        shape = (r.Nkl, case["Nj"])
        if run["coeff"] == "fixture":
            Ap, Am, A0 = (a.reshape(shape) for a in fixture_coefficients(r.M))
        else:
            base = sum(ord(ch) for ch in run["case"]) + 200
            Ap, Am, A0 = (seeded(shape, base + i, 1e-3) for i in (1, 2, 3))
        lib.wvref_destroy(r.h)
        v = {**BASE, **{k: case[k] for k in case if k in BASE}}
        sizes = (ctypes.c_uint64 * 4)(case["Nx"], case["Ny"], case["Nz"], case["Nj"])
        values = (ctypes.c_double * 9)(case["Lx"], case["Ly"], case["Lz"], v["N0"], v["rho0"], v["g"],
                                       v["planetaryRadius"], v["rotationRate"], case["latitude"])
        flags = (ctypes.c_uint8 * 2)(int(case["isHydrostatic"]), int(case["shouldAntialias"]))
        G = run["groups"]
        T = run["tracers"]
        ints = lambda vals: (ctypes.c_int * max(1, len(vals)))(*vals)
        dbls = lambda vals: (ctypes.c_double * max(1, len(vals)))(*vals)
        xs = [a for g in G for a in g["x"]]
        ys = [a for g in G for a in g["y"]]
        zs = [a for g in G for a in g["z"]]
        h = ctypes.c_void_p()
        rc = lib.wvref_system_create(sizes, values, flags, run["schedule"], len(G), ints([len(g["x"]) for g in G]),
                                     ints([int(g["xy_only"]) for g in G]), ints([int(g["spline"]) for g in G]),
                                     dbls([g["tol_h"] for g in G]), dbls([g["tol_v"] for g in G]), dbls(xs), dbls(ys),
                                     dbls(zs), len(T), ints([int(t["antialias"]) for t in T]), dbls([t["tol"] for t in T]),
                                     ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"system create failed: {rc} {lib.wvref_system_message(h)}")
        extra = []
        for g in G:
            extra += [np.array(g["x"]), np.array(g["y"])] + ([] if g["xy_only"] else [np.array(g["z"])])
        tracer_fields = [tracer_field(case, t["scale"]) for t in T]
        extra += [f.ravel() for f in tracer_fields]
        ex = np.ascontiguousarray(np.concatenate(extra))
        assert ex.size == lib.wvref_system_extra(h)
        Ap, Am, A0 = (np.ascontiguousarray(a) for a in (Ap, Am, A0))
        F = [np.zeros(shape, np.complex128) for _ in range(3)]
        er = np.zeros_like(ex)
        chk = lambda rc: (_ for _ in ()).throw(RuntimeError(lib.wvref_system_message(h).decode())) if rc else None
        chk(lib.wvref_system_rhs(h, ctypes.c_double(run["t"]), ctypes.c_double(run["t0"]), P(Ap), P(Am), P(A0), P(ex),
                                 P(F[0]), P(F[1]), P(F[2]), P(er)))
        Kp, Km, K0, kex = Ap.copy(), Am.copy(), A0.copy(), ex.copy()
        tt = ctypes.c_double(run["t"])
        chk(lib.wvref_system_rk4(h, P(Kp), P(Km), P(K0), P(kex), ctypes.byref(tt), ctypes.c_double(run["t0"]),
                                 ctypes.c_double(run["dt"]), ctypes.c_int(run["steps"])))
        rk = run["rk23"]
        Rp, Rm, R0, rex = Ap.copy(), Am.copy(), A0.copy(), ex.copy()
        t23 = ctypes.c_double(run["t"])
        counts = (ctypes.c_ulonglong * 4)()
        nxt = ctypes.c_double()
        steps = np.zeros(4096)
        chk(lib.wvref_system_rk23(h, (ctypes.c_double * 6)(*rk["opts"]), P(Rp), P(Rm), P(R0), P(rex), ctypes.byref(t23),
                                  ctypes.c_double(run["t0"]), ctypes.c_double(rk["final"]), ctypes.c_double(rk["initial"]),
                                  counts, ctypes.byref(nxt), P(steps), ctypes.c_int(4096)))
        counts = np.array(list(counts), np.uint64)
        lib.wvref_system_destroy(h)
        out.update({f"{key}_Ap": Ap, f"{key}_Am": Am, f"{key}_A0": A0, f"{key}_extra": ex, f"{key}_t": run["t"],
                    f"{key}_t0": run["t0"], f"{key}_Fp": F[0], f"{key}_Fm": F[1], f"{key}_F0": F[2], f"{key}_rhs_extra": er,
                    f"{key}_dt": run["dt"], f"{key}_steps": run["steps"], f"{key}_Kp": Kp, f"{key}_Km": Km, f"{key}_K0": K0,
                    f"{key}_k_extra": kex, f"{key}_k_t": tt.value, f"{key}_rk23_final": rk["final"],
                    f"{key}_rk23_initial": rk["initial"], f"{key}_rk23_opts": np.array(rk["opts"]), f"{key}_Rp": Rp,
                    f"{key}_Rm": Rm, f"{key}_R0": R0, f"{key}_r_extra": rex, f"{key}_r_t": t23.value,
                    f"{key}_r_counts": counts, f"{key}_r_next": nxt.value, f"{key}_r_steps": steps[:int(counts[0])].copy()})
        print(f"system {key}: rk23 counts {counts.tolist()}")
    with open(os.path.join(HERE, "system_runs.json"), "w") as fh:
        json.dump(SYSTEM_RUNS, fh, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "system.npz"), **out)


# Fixed-step RK4 advanceToTime with a final partial step and retained dense
# output, through the reference's WVFixedStepRK4 ({retainDenseOutput = true}).
RK4_DENSE_RUNS = {
    "odd": dict(case="odd_15x13x9", damping=False, t=100.0, t0=3.0, final=165.0, dt=20.0, theta=0.37),
    "hd": dict(case="hydro_damp_12x10x11", damping=True, t=10.0, t0=1.0, final=40.0, dt=12.5, theta=0.81),
}


def make_rk4_dense(lib):
    out = {}
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    for key, run in RK4_DENSE_RUNS.items():
        case = CASES[run["case"]]
        r = Ref(lib, case)
        shape = (r.Nkl, case["Nj"])
        base = sum(ord(ch) for ch in run["case"]) + 300
        Ap, Am, A0 = (seeded(shape, base + i, 1e-3) for i in (1, 2, 3))
        Kp, Km, K0 = Ap.copy(), Am.copy(), A0.copy()
        tt = ctypes.c_double(run["t"])
        dense = np.zeros((3,) + shape, np.complex128)
        interval = np.zeros(2)
        # the last step runs from the largest multiple of dt below final (here a partial step)
        n_full = int((run["final"] - run["t"]) // run["dt"])
        t_last = run["t"] + n_full * run["dt"]
        if t_last >= run["final"]:
            t_last -= run["dt"]
        dense_time = t_last + run["theta"] * (run["final"] - t_last)
        r.check(lib.wvref_rk4_dense(r.h, P(Kp), P(Km), P(K0), ctypes.byref(tt), ctypes.c_double(run["t0"]),
                                    ctypes.c_double(run["final"]), ctypes.c_double(run["dt"]), ctypes.c_double(dense_time),
                                    P(dense), P(interval)))
        out.update({f"{key}_Ap": Ap, f"{key}_Am": Am, f"{key}_A0": A0, f"{key}_t": run["t"], f"{key}_t0": run["t0"],
                    f"{key}_final": run["final"], f"{key}_dt": run["dt"], f"{key}_damping": run["damping"],
                    f"{key}_Kp": Kp, f"{key}_Km": Km, f"{key}_K0": K0, f"{key}_tout": tt.value,
                    f"{key}_dense_time": dense_time, f"{key}_dense": dense, f"{key}_interval": interval})
        lib.wvref_destroy(r.h)
        print(f"rk4 dense {key}: interval {interval.tolist()} t = {tt.value}")
    np.savez_compressed(os.path.join(HERE, "rk4_dense.npz"), **out)


if __name__ == "__main__":
    root = next((a for a in sys.argv[1:] if not a.startswith("--")), None)
    if "--rk23" in sys.argv:
        make_rk23(load_lib(root))
    elif "--system" in sys.argv:
        make_system(load_lib(root))
    elif "--rk4-dense" in sys.argv:
        make_rk4_dense(load_lib(root))
    else:
        main()
        make_rk23(load_lib(root))
        make_system(load_lib(root))
        make_rk4_dense(load_lib(root))

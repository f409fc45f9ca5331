"""Shared helpers: golden cases and tolerances."""
import json
import os

import numpy as np

import wv_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# Plain-FP64 parity gate of the reference's compiled backend
# (@WVCompiledConstantStratificationBackend/WVCompiledConstantStratificationBackend.m:152).
FP64_REL_TOL = 1e-12


def golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as fh:
        return json.load(fh)


def config_from_case(cf):
    return O.Config(Nx=cf["Nx"], Ny=cf["Ny"], Nz=cf["Nz"], Nj=cf["Nj"], Lx=cf["Lx"], Ly=cf["Ly"], Lz=cf["Lz"],
                    N0=cf["N0"], rho0=cf["rho0"], g=cf["g"], planetaryRadius=cf["planetaryRadius"],
                    rotationRate=cf["rotationRate"], latitude=cf["latitude"], isHydrostatic=cf["isHydrostatic"],
                    shouldAntialias=cf["shouldAntialias"])


def load_golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def rel_err(a, b):
    """max |a-b| / max |b| (the reference's relative-error convention)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = float(np.max(np.abs(b))) if b.size else 0.0
    num = float(np.max(np.abs(a - b))) if b.size else 0.0
    return num / den if den > 0 else num


def state_components_close(got, golden, keys, tol):
    """Per-component parity of a state (Kp, Km, K0, ...) against golden arrays:
    a component whose golden values stay below 1e-6 of the state's largest
    coefficient is accumulated rounding (the single-wave case's A0 starts at
    zero and ends at 3e-10 of Ap, its digits set by the summation order) and is
    gated relative to the state; every other component relative to itself.
    Returns the failing keys."""
    scale = max(float(np.max(np.abs(golden[k]))) for k in keys)
    bad = []
    for a, k in zip(got, keys):
        ref = golden[k]
        if not np.any(ref):
            continue
        if float(np.max(np.abs(ref))) < 1e-6 * scale:
            if float(np.max(np.abs(np.asarray(a) - ref))) > tol * scale:
                bad.append(k)
        elif rel_err(a, ref) > tol:
            bad.append(k)
    return bad


def parity_tolerance(floor):
    """Parity gate for states where the FP64 noise floor of the computation
    (two valid orderings of the oracle) exceeds the reference's 1e-12 gate:
    within 3x that measured floor, never looser than needed."""
    return max(FP64_REL_TOL, 3.0 * floor)


# Adaptive RK23 fixture runs (tests/golden/rk23.npz) and the golden case each uses.
RK23_RUNS = {"odd": "odd_15x13x9", "wave": "wave_16x16x9", "hd": "hydro_damp_12x10x11"}


def rk23_run(key):
    """Inputs and reference outputs of one RK23 fixture run."""
    g = load_golden("rk23")
    cf = golden_cases()[RK23_RUNS[key]]
    o = g[f"{key}_opts"]
    options = dict(rtol=float(o[0]), atol_scale=float(o[1]), safety=float(o[2]), floor=float(o[3]),
                   max_factor=float(o[4]), max_step=float(o[5]))
    out = {n: g[f"{key}_{n}"] for n in ("Ap", "Am", "A0", "Kp", "Km", "K0", "diag", "counts", "hashes", "dense")}
    out.update({n: float(g[f"{key}_{n}"]) for n in ("t", "t0", "final", "initial", "tout", "next", "dense_time")})
    return cf, options, out


def system_run(key):
    """Inputs and reference outputs of one integrated-observer fixture run
    (tests/golden/system.npz): (case config, run spec, arrays)."""
    with open(os.path.join(GOLDEN, "system_runs.json")) as fh:
        run = json.load(fh)[key]
    g = load_golden("system")
    arrays = {k[len(key) + 1:]: g[k] for k in g.files if k.startswith(key + "_")}
    return golden_cases()[run["case"]], run, arrays


def system_observers(run):
    """Oracle particle groups and tracers of a fixture run."""
    groups = [O.ParticleGroup(x=np.array(g["x"]), y=np.array(g["y"]), z=np.array(g["z"]), xy_only=g["xy_only"],
                              spline=g["spline"], horizontal_tolerance=g["tol_h"], vertical_tolerance=g["tol_v"])
              for g in run["groups"]]
    tracers = [O.Tracer(antialias=t["antialias"], tolerance=t["tol"]) for t in run["tracers"]]
    return groups, tracers


def split_extra(desc, groups, tracers, extra):
    """Packed additional state -> list of blocks (particles 1-D, tracers (Nz, Ny, Nx))."""
    c = desc.c
    out, off = [], 0
    for g in groups:
        n = len(g.x)
        for _ in range(2 if g.xy_only else 3):
            out.append(np.asarray(extra[off:off + n]))
            off += n
    R = c.Nx * c.Ny * c.Nz
    for _ in tracers:
        out.append(np.asarray(extra[off:off + R]).reshape(c.Nz, c.Ny, c.Nx))
        off += R
    assert off == len(extra)
    return out


def rk4_dense_run(key):
    """Inputs and reference outputs of one RK4 advanceToTime / dense-output run
    (tests/golden/rk4_dense.npz)."""
    g = load_golden("rk4_dense")
    cfg = {"odd": "odd_15x13x9", "hd": "hydro_damp_12x10x11"}[key]
    return golden_cases()[cfg], {k[len(key) + 1:]: g[k] for k in g.files if k.startswith(key + "_")}

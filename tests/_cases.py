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


def parity_tolerance(floor):
    """Parity gate for states where the FP64 noise floor of the computation
    (two valid orderings of the oracle) exceeds the reference's 1e-12 gate:
    within 3x that measured floor, never looser than needed."""
    return max(FP64_REL_TOL, 3.0 * floor)

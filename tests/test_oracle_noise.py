"""The oracle's two vertical orderings agree to FP64 rounding on the golden
cases (so the dense ordering is a valid second evaluation), and the measured
noise floor of the flux is what the parity gate for large states builds on."""
import numpy as np

import wv_oracle as O
from _cases import FP64_REL_TOL, config_from_case, golden_cases, load_golden, rel_err


def test_dense_ordering_matches_reference_golden():
    for name, cf in golden_cases().items():
        d = O.build_descriptor(config_from_case(cf))
        g = load_golden(name)
        with O.dense_vertical():
            F = O.nonlinear_flux(d, g["Ap"], g["Am"], g["A0"], float(g["t"]), float(g["t0"]))
        for got, key in zip(F, ("Fp", "Fm", "F0")):
            assert rel_err(got, g[key]) <= FP64_REL_TOL, (name, key)


def test_noise_floor_is_small_but_nonzero_on_spectrum_state():
    c = O.Config(Nx=32, Ny=32, Nz=17, Nj=10, Lx=200e3, Ly=200e3, Lz=4000.0, latitude=33.0)
    d = O.build_descriptor(c)
    A = O.spectrum_state(d, seed=7, urms=0.1)
    _, floors = O.noise_floor(O.nonlinear_flux, d, *A, 100.0, 0.0)
    assert all(0.0 <= f < 1e-9 for f in floors)

"""The oracle against its committed regression fixtures (tests/golden/,
written by tests/golden/make_golden.py): an r2c in the reference's layout and
a 10-step 16^3 run with a 12-bead chain and Philox noise.  The tolerance
allows for libm differences between host machines; any change to the
oracle's arithmetic shows up far above it."""
import os

import numpy as np

from oracle import oracle as OR
from oracle.oracle import Oracle
from tests.golden.make_golden import step_case
from tests.helpers import rel_err

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_cases.npz")


def load():
    return np.load(GOLDEN)


def test_fft_fixture():
    g = load()
    assert rel_err(OR.fft_r2c(g["fft_in"]), g["fft_out"]) < 1e-13


def test_step_fixture():
    g = load()
    chains = (g["x0"], g["tags"], g["mol"], g["types"])
    phi, x, ux, f, im = step_case(Oracle(), g["phi0"], chains)
    assert rel_err(phi, g["phi"]) < 1e-13
    assert rel_err(ux, g["ux"]) < 1e-13 and rel_err(f, g["f"]) < 1e-11
    assert np.array_equal(im, g["images"])

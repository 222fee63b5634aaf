"""The oracle against the reference's own code.

tests/golden/ref_<scenario>.npz hold final states of the reference's sources
(compiled unmodified against stand-ins of MPI, FFTW, Eigen, fftw_arr and
beadrodpmer, oracle/refpin) on the scenarios of tests/ref_scenarios.py,
written by tests/golden/make_ref_golden.py.  Replaying each scenario on the
FP64 oracle must give:
  phi, chempot and the three gradient fields within 1e-12 relative (the two
  sides' discrete Fourier transforms round differently);
  owned-bead positions within 1e-12 of the largest coordinate, unwrapped
  positions and forces within 1e-10 relative, image flags equal;
  the same number of neighbor builds and Flory-Huggins reflections;
  the half bead list and the grid list equal as sets of (tag, tag, image) and
  (node, tag, image), bit for bit.
"""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from tests import ref_scenarios as RS
from tests.helpers import canon_grid, canon_half, rel_err

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture(name):
    return np.load(os.path.join(GOLDEN, "ref_%s.npz" % name))


def replay(driver, name, steps=None):
    sc = RS.SCENARIOS[name]
    fx = fixture(name)
    beads = (fx["in_tags"], fx["in_mol"], fx["in_types"], fx["in_x"])
    RS.apply(driver, sc, beads)
    driver.setup()
    driver.run(sc["steps"] if steps is None else steps)
    return fx


def check_state(d, fx, field_tol, bead_tol, grads=True, chempot=True):
    assert rel_err(d.grid_get("phi"), fx["phi"]) < field_tol
    if chempot:
        assert rel_err(d.grid_get("chempot"), fx["chempot"]) < field_tol
    if grads:
        for f in ("gradx", "grady", "gradz"):
            assert rel_err(d.grid_get(f), fx[f]) < field_tol, f
    c = d.counters()
    nowned, timestep, ncalls, less, great = (int(v) for v in fx["counters"])
    assert (c["num_less_zero"], c["num_great_zero"]) == (less, great)
    assert c["timestep"] == timestep
    if nowned:  # with no beads the reference still counts its set-up build; the lists are empty
        assert c["neighbor_calls"] == ncalls
        x, ux, f, img = d.atoms_get()
        assert np.abs(x - fx["x"]).max() <= bead_tol * np.abs(fx["x"]).max()
        assert np.abs(ux - fx["ux"]).max() <= 100 * bead_tol * np.abs(fx["ux"]).max()
        assert rel_err(f, fx["f"]) < 100 * bead_tol
        assert np.array_equal(img, fx["images"])
        assert canon_half(d.half_list()) == canon_half(fx["half_list"])
        assert canon_grid(d.grid_list()) == canon_grid(fx["grid_list"])


def replay_computes(d, name, fx, tol):
    """compute pair after the last step (compute_pair.cpp:43-85): the style's
    per-bead forces, and the chempot array it leaves (the reference's compute
    re-runs the pair, adding that style's deposit to chempot once more)."""
    if not RS.SCENARIOS[name]["compute_pair"]:
        return
    got = d.compute_pair("gridatom")
    want = fx["compute_cpair"].reshape(-1, 3)
    assert rel_err(got, want) < tol
    assert rel_err(d.grid_get("chempot"), fx["chempot"]) < tol


@pytest.mark.parametrize("name", sorted(RS.SCENARIOS))
def test_oracle_matches_the_reference(name):
    o = Oracle()
    fx = replay(o, name)
    with_compute = RS.SCENARIOS[name]["compute_pair"]
    check_state(o, fx, 1e-12, 1e-12, chempot=not with_compute)
    replay_computes(o, name, fx, 1e-12)


def test_scenarios_exercise_what_they_claim():
    """Each fixture holds the behaviour its scenario is there for."""
    assert int(fixture("rebuilds")["counters"][2]) >= 2            # a neighbor rebuild
    c = fixture("field_reflections")["counters"]
    assert int(c[3]) > 0 and int(c[4]) > 0                          # reflections on both sides
    assert fixture("aniso_box")["phi"].shape == (32, 16, 16)        # Nz, Ny, Nx
    assert "compute_cpair" in fixture("ljish_linear_pair").files    # per-bead forces of one style
    for name in RS.SCENARIOS:
        fx = fixture(name)
        if RS.SCENARIOS[name]["nbeads"]:
            assert len(fx["grid_list"]) > 0 and len(fx["half_list"]) > 0

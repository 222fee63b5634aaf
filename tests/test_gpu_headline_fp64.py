"""The FP64 GPU path against the FP64 oracle at the headline size.

256^3 grid on a box of side 256, phi = 0.4 + U(-0.01, 0.01), chi = 3;
64 semiflexible chains of 500 beads (32,000 beads) laid as random walks of
bond length 1; WCA lj/cut, gridatom/gaussian coupling of width 1, bead
kT = 1.  The field noise and the bead noise are the same Philox streams on
both sides (generated from the seeds, so both runs receive identical noise).
After 20 steps, which include neighbor rebuilds, per-node phi and per-bead
positions agree within 1e-10 relative, image flags, reflection counts and
the number of neighbor builds are equal, and both neighbor lists (bead
pairs and grid-node/bead pairs) are equal as sets, bit for bit.

This follows the reference's step (integrate.cpp:105-203) at full size;
the oracle's grid loops run on every host thread (bit-identical to one).
"""
import numpy as np
import pytest

from oracle import oracle as OR
from oracle.oracle import Oracle
from phafd_gb300 import workloads as W
from tests.helpers import canon_grid, canon_half, rel_err

pytestmark = pytest.mark.gpu

STEPS = 20


def test_headline_workload_fp64_matches_oracle(gpu_lib):
    from phafd_gb300.gpu import PhafdGPU
    cfg = W.CONFIGS["256cube_32kbeads"]
    OR.set_threads(OR.host_threads())
    o = Oracle()
    g = PhafdGPU(precision=64, schedule="resident")
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(STEPS)
    po, pg = o.grid_get("phi"), g.grid_get("phi")
    assert rel_err(pg, po) < 1e-10
    xo, uxo, fo, imo = o.atoms_get()
    xg, uxg, fg, img = g.atoms_get()
    assert len(xo) == 32000
    assert np.array_equal(imo, img)
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()
    assert np.abs(uxg - uxo).max() < 1e-10 * np.abs(uxo).max()
    assert rel_err(fg, fo) < 1e-9
    co, cg = o.counters(), g.counters()
    assert cg["neighbor_calls"] == co["neighbor_calls"]
    assert co["neighbor_calls"] >= 2  # the set-up build and at least one rebuild
    assert (cg["num_less_zero"], cg["num_great_zero"]) == (co["num_less_zero"], co["num_great_zero"])
    # total concentration
    assert abs(pg.sum() - po.sum()) < 1e-10 * abs(po.sum())
    # the lists of the last build, as sets
    assert canon_half(g.half_list()) == canon_half(o.half_list())
    assert canon_grid(g.grid_list()) == canon_grid(o.grid_list())
    g.close()

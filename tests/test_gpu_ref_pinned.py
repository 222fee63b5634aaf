"""The FP64 GPU path against the reference's own code.

Replays the scenarios of tests/ref_scenarios.py on the CUDA path (FP64, the
reference's mt19937 field noise, its one-rank z ghosts) and compares with
the final states of the reference's sources in tests/golden/ref_*.npz
(see tests/test_ref_pinned.py for how they were made):
  reference schedule: phi, chempot, the three gradient fields within 1e-10
  relative; owned-bead positions within 1e-10 of the largest coordinate,
  forces within 1e-8 relative; image flags, neighbor builds, reflection
  counts and both lists (as sets) equal;
  resident schedule (which carries the spectrum across steps and keeps the
  gradient of the current phi): the same except the gradient fields;
  both: the step-start gradient fields (what the reference's gradphi dump
  attributes hold) within 1e-10, and compute pair's per-bead forces and the
  chempot it leaves within 1e-10.
"""
import pytest

from tests import ref_scenarios as RS
from tests.helpers import rel_err
from tests.test_ref_pinned import check_state, replay, replay_computes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("schedule", ["reference", "resident"])
@pytest.mark.parametrize("name", sorted(RS.SCENARIOS))
def test_gpu_matches_the_reference(gpu_lib, name, schedule):
    from phafd_gb300.gpu import PhafdGPU
    g = PhafdGPU(precision=64, schedule=schedule)
    g.set_keep_chempot(True)
    with_compute = RS.SCENARIOS[name]["compute_pair"]
    if with_compute:
        g.set_pair_snapshot(True)
    fx = replay(g, name)
    check_state(g, fx, 1e-10, 1e-10, grads=schedule == "reference", chempot=not with_compute)
    # the gradient the reference's arrays hold after a step, in either schedule
    for f in ("gradx", "grady", "gradz"):
        assert rel_err(g.grid_get(f + "_step_start"), fx[f]) < 1e-10, f
    replay_computes(g, name, fx, 1e-10)
    g.close()

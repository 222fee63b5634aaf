"""run_until_touching on the GPU against the oracle (FP64, noise off): same
steps taken, same events."""
import pytest

from oracle.oracle import Oracle
from phafd_gb300.gpu import PhafdGPU
from tests.test_touching_oracle import distances, scene, touch_between

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cont,delay,q", [(False, 0, 0.3), (True, 0, 0.5), (True, 3, 0.5), (True, 10, 0.2)])
def test_touching_matches_oracle(gpu_lib, cont, delay, q):
    n = 60
    touch = touch_between(distances(n), q)
    want = scene(Oracle()).run_until_touching(n, touch, cont, delay)
    got = scene(PhafdGPU(precision=64, schedule="resident")).run_until_touching(n, touch, cont, delay)
    assert got == want


def test_touching_then_plain_run_continues(gpu_lib):
    """After run_until_touching the context runs plain steps (the check is off)."""
    g = scene(PhafdGPU(precision=64, schedule="resident"))
    o = scene(Oracle())
    assert g.run_until_touching(5, 0.0, True, 0) == o.run_until_touching(5, 0.0, True, 0)
    g.run(7)
    o.run(7)
    import numpy as np
    xg, xo = g.atoms_get()[0], o.atoms_get()[0]
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()

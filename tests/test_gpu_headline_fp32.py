"""The FP32 production path against the FP64 oracle at the headline size.

256^3 grid (box 256), phi = 0.4 + U(-0.01, 0.01), chi = 3, 64 chains x 500
beads (32,000 beads), bead kT = 1, the same Philox field and bead noise on
both sides, 50 steps (the bench's precision window).  The FP32 path is held
to a relative shell-averaged S(k) error of at most 1e-5 against the oracle,
with total concentration kept to FP32 rounding and bead positions within
1e-6 relative, with its default stages relative to the mean of phi (the
transforms) and with the Flory-Huggins part centered too.  With both
switched off (phafd_set_fp32_centering(ctx, 0)), the same run misses that
bound: the test shows what the centering buys.
"""
import numpy as np
import pytest

from oracle import oracle as OR
from oracle.oracle import Oracle
from phafd_gb300 import workloads as W
from tests.helpers import sk_rel_err

pytestmark = pytest.mark.gpu

STEPS = 50


@pytest.fixture(scope="module")
def oracle_run():
    cfg = W.CONFIGS["256cube_32kbeads"]
    OR.set_threads(OR.host_threads())
    o = Oracle()
    chains = W.apply(o, cfg)
    o.setup()
    o.run(STEPS)
    out = (o.grid_get("phi"), o.atoms_get()[0], chains)
    del o
    return out


def gpu_run(chains, centering):
    from phafd_gb300.gpu import PhafdGPU
    cfg = W.CONFIGS["256cube_32kbeads"]
    g = PhafdGPU(precision=32, schedule="resident")
    W.apply(g, cfg, chains=chains)
    if centering is not None:
        g.set_fp32_centering(fh=centering, fft=centering)
    g.setup()
    g.run(STEPS)
    out = g.grid_get("phi"), g.atoms_get()[0]
    g.close()
    return out


@pytest.mark.parametrize("centering", [None, True])  # the default (transforms), and both stages
def test_headline_workload_fp32_sk_within_1e5_of_oracle(gpu_lib, oracle_run, centering):
    po, xo, chains = oracle_run
    pg, xg = gpu_run(chains, centering)
    assert sk_rel_err(pg, po) < 1e-5
    assert abs(pg.mean() - po.mean()) < 1e-7
    assert np.abs(xg - xo).max() < 1e-6 * np.abs(xo).max()


def test_headline_workload_fp32_without_centering_misses_the_bound(gpu_lib, oracle_run):
    po, _, chains = oracle_run
    pg, _ = gpu_run(chains, False)
    assert sk_rel_err(pg, po) > 1e-5

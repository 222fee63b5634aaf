"""Ragged ensemble: replicas enqueued together give the same fields as the
same replicas run one after another."""
import numpy as np
import pytest

from phafd_gb300 import workloads as W
from phafd_gb300.ensemble import Ensemble, ensemble_configs
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def test_ensemble_matches_sequential_runs(gpu_lib):
    cfgs = ensemble_configs(nrep=3, seed=7, sizes=(32, 64, 96))
    for c in cfgs:  # keep it small
        c["nchains"] = 4
        c["chain_len"] = 50
    chains = [W.random_walk_chains(c["nchains"], c["chain_len"], c["origin"], c["L"], c["chain_seed"]) for c in cfgs]
    ens = Ensemble(cfgs, precision=64, chains=chains)
    ens.run(10)
    together = [g.grid_get("phi") for g in ens.replicas]
    ens.close()
    from phafd_gb300.gpu import PhafdGPU
    for cfg, ch, phi in zip(cfgs, chains, together):
        g = PhafdGPU(precision=64)
        W.apply(g, cfg, chains=ch)
        g.setup()
        g.run(10)
        assert rel_err(phi, g.grid_get("phi")) < 1e-12
        g.close()

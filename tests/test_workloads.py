"""Host-side workload definitions: the algorithmic bytes per step that the
roofline divides by, the ragged ensemble's draws, and the chain generator's
geometry (no GPU)."""
import numpy as np

from phafd_gb300 import workloads as W
from phafd_gb300.ensemble import ensemble_configs


def test_algorithmic_bytes_per_step():
    # B_step = 6 s N + 10 s N_c + N_b (5 s P + 24 s), P = 4.19
    cfg = W.CONFIGS["256cube_32kbeads"]
    n = 256
    N, Nc, Nb = n ** 3, (n // 2 + 1) * n * n, 32000
    for s, total_gb in ((4, 0.747), (8, 1.493)):
        b = W.algorithmic_bytes_per_step(cfg, s)
        assert b == 6 * s * N + 10 * s * Nc + Nb * (5 * s * 4.19 + 24 * s)
        assert abs(b / 1e9 - total_gb) < 1e-3
    big = W.algorithmic_bytes_per_step(W.CONFIGS["512cube_1Mbeads"], 4)
    assert abs(big / 1e9 - 6.096) < 1e-3  # 5.92 GB of grid traffic + the million beads' terms


def test_ensemble_draws():
    cfgs = ensemble_configs(48)
    assert len(cfgs) == 48
    assert {c["n"] for c in cfgs} <= {96, 128, 160}
    for c in cfgs:
        nb = c["nchains"] * c["chain_len"]
        assert 100 <= c["chain_len"] <= 400
        assert 2000 - c["chain_len"] < nb <= 20000
        assert 2.2 <= c["chi"] <= 3.5 and 0.3 <= c["phi0"] <= 0.5
        assert c["L"] == float(c["n"]) and c["origin"] == -c["n"] / 2.0
    assert len({c["grid_seed"] for c in cfgs}) == 48  # one seed per replica
    assert ensemble_configs(48) == cfgs  # seeded


def test_random_walk_chains_geometry():
    x, tags, mol, types = W.random_walk_chains(3, 40, -16.0, 32.0, 11)
    assert x.shape == (120, 3) and list(tags) == list(range(1, 121))
    assert list(np.unique(mol)) == [0, 1, 2] and not types.any()
    for c in range(3):
        seg = x[40 * c: 40 * (c + 1)]
        assert np.allclose(np.linalg.norm(np.diff(seg, axis=0), axis=1), 1.0)  # bond length 1

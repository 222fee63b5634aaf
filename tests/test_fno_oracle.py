"""The CPU oracle of the learned propagator: its manual backward pass agrees
with finite differences of its forward pass (FP64, no rounding)."""
import numpy as np

from oracle.fno_oracle import FNOOracle
from phafd_gb300.fno import init_params, layout, param_count

SHAPE = (16, 16, 16)
NORM = [0.45, 0.05, 0.0, 1.0, 3.0, 0.3, 1.0, 0.0]


def scene(seed=1):
    rng = np.random.default_rng(seed)
    phi = 0.45 + 0.05 * rng.standard_normal(SHAPE)
    rho = np.abs(rng.standard_normal(SHAPE)) * (rng.random(SHAPE) < 0.05)
    tgt = 0.3 * rng.standard_normal(SHAPE)
    return phi, rho, tgt


def loss_of(p, phi, rho, tgt):
    return FNOOracle(p, SHAPE, NORM, bf=False).loss_and_grad(phi, rho, 3.1, tgt)


def test_param_layout_is_contiguous():
    off = sorted(layout().values(), key=lambda t: t[0])
    pos = 0
    for o, shp in off:
        assert o == pos
        pos += int(np.prod(shp))
    assert pos == param_count()


def test_backward_matches_finite_differences():
    phi, rho, tgt = scene()
    p = init_params(3, out_scale=1.0).astype(np.float64)
    _, g = loss_of(p, phi, rho, tgt)
    gv = FNOOracle.flat(g)
    rng = np.random.default_rng(7)
    h = 1e-6
    groups = [None, "P", "W0", "R1", "b2", "R3", "Q1", "q2"]
    for name in groups:
        d = np.zeros(p.size)
        if name is None:
            d[:] = rng.standard_normal(p.size)
        else:
            o, shp = layout()[name]
            n = int(np.prod(shp))
            d[o:o + n] = rng.standard_normal(n)
        lp, _ = loss_of(p + h * d, phi, rho, tgt)
        lm, _ = loss_of(p - h * d, phi, rho, tgt)
        fd = (lp - lm) / (2 * h)
        an = gv @ d
        assert abs(fd - an) <= 1e-4 * abs(fd) + 1e-12, (name, fd, an)


def test_correction_carries_no_mass():
    phi, rho, _ = scene(2)
    p = init_params(4, out_scale=1.0).astype(np.float64)
    corr = FNOOracle(p, SHAPE, NORM, bf=True).correction(phi, rho, 3.0)
    assert abs(corr.mean()) < 1e-12 * max(1.0, np.abs(corr).max())

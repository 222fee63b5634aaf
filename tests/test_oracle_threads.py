"""The oracle's threaded grid loops give bit-identical results to one thread:
FFT round trips at power-of-two and mixed-radix sizes, and whole steps with
each noise mode (the reference generator's bulk update stays serial)."""
import numpy as np
import pytest

from oracle import oracle as OR
from oracle.oracle import Oracle
from phafd_gb300 import workloads as W


@pytest.fixture
def threads():
    yield OR.set_threads
    OR.set_threads(1)


@pytest.mark.parametrize("shape", [(32, 32, 32), (20, 12, 18), (3, 5, 6)])
def test_fft_bit_identical(threads, shape):
    rng = np.random.default_rng(1)
    phi = rng.standard_normal(shape)
    out = []
    for t in (1, 3, 8):
        threads(t)
        c = OR.fft_r2c(phi)
        out.append((c, OR.fft_c2r(c, shape)))
    for c, r in out[1:]:
        assert np.array_equal(c, out[0][0]) and np.array_equal(r, out[0][1])


@pytest.mark.parametrize("noise", ["off", "reference", "philox"])
def test_steps_bit_identical(threads, noise):
    cfg = dict(W.CONFIGS["32cube_64beads"], field_noise=noise, bead_temp=1.0 if noise == "philox" else 0.0,
               dt=5e-4, phi0=0.5, amp=1.1)  # phi0 + amp*U(-1/2, 1/2) leaves (0, 1): reflections count
    res = []
    for t in (1, 5):
        threads(t)
        o = Oracle()
        W.apply(o, cfg)
        o.setup()
        o.run(8)
        res.append((o.grid_get("phi"), o.atoms_get()[1], o.counters()))
    assert np.array_equal(res[0][0], res[1][0], equal_nan=True)
    assert np.array_equal(res[0][1], res[1][1], equal_nan=True)
    assert res[0][2] == res[1][2]
    assert res[0][2]["num_less_zero"] + res[0][2]["num_great_zero"] > 0

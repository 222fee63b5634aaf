"""grid_populate flat_interface / sphere (grid.cpp:136-166, 310-425) on the
oracle, pinned against independent restatements: the flat interface draws the
same mt19937 stream as the constant concentration with the same seed, and the
sphere follows the reference's loops with the C library's tanh and sqrt."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle, OracleError

SHAPE = (12, 10, 16)  # nz, ny, nx
LO, L = [-8.0, -5.0, -6.0], [16.0, 10.0, 12.0]


def oracle(populate):
    o = Oracle()
    o.domain(LO, L)
    o.grid_style(SHAPE[2], SHAPE[1], SHAPE[0])
    populate(o)
    return o.grid_get("phi")


def test_flat_interface_matches_constant_stream():
    avg, var, hi, lo, seed = 0.45, 0.05, 0.8, 0.2, 7
    got = oracle(lambda o: o.grid_populate_flat_interface(avg, var, hi, lo, seed))
    noise = oracle(lambda o: o.grid_populate_constant(0.0, var, seed))  # 0 + var U = var U exactly
    nx = SHAPE[2]
    x = np.arange(nx) * (L[0] / nx) + LO[0]
    inside = (x - LO[0]) < (avg - lo) / (hi - lo) * L[0]
    base = np.where(inside, hi, lo)[None, None, :]
    assert np.array_equal(got, base + noise)
    assert 0 < inside.sum() < nx


def sphere_restated(radius, width, hi, av):
    nz, ny, nx = SHAPE
    h = [L[0] / nx, L[1] / ny, L[2] / nz]
    f = np.empty(SHAPE)
    integral = 0.0
    for i in range(nz):
        z = i * h[2] + LO[2]
        for j in range(ny):
            y = j * h[1] + LO[1]
            for k in range(nx):
                x = k * h[0] + LO[0]
                f[i, j, k] = math.tanh((-math.sqrt(x * x + y * y + z * z) + radius) / width)
                integral += f[i, j, k]
    integral *= h[0] * h[1] * h[2]
    ifrac = integral / (L[0] * L[1] * L[2])
    lo = (2 * av - hi * (1 + ifrac)) / (1 - ifrac)
    return 0.5 * (hi - lo) * f + 0.5 * (hi + lo), lo


def test_sphere_matches_restatement():
    radius, width, hi, av = 3.5, math.sqrt(2.0), 0.9, 0.3
    got = oracle(lambda o: o.grid_populate_sphere(radius, width, hi, av))
    want, lo = sphere_restated(radius, width, hi, av)
    assert np.abs(got - want).max() <= 4e-16
    assert abs(got.mean() - av) < 1e-12  # the outer value fixes the volume average
    assert got.max() <= hi and got.min() >= lo - 1e-15


@pytest.mark.parametrize("args,msg", [
    ((5.0, 1.0, 0.9, 0.3), "radius > domain"),
    ((3.5, 1.0, 0.9, 0.01), "too small"),
    ((3.5, 1.0, 0.9, 0.95), "too large"),
])
def test_sphere_errors(args, msg):
    with pytest.raises(OracleError, match=msg):
        oracle(lambda o: o.grid_populate_sphere(*args))

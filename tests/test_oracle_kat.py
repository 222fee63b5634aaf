"""Known-answer tests that pin the oracle (the reference ships none).

* linear Model-B growth rate of a small sinusoid (noise off)
* exact conservation of the k = 0 mode
* zero gridatom force in a constant field
* analytic LJ force
* neighbor lists against brute-force O(N^2) sets
* Hermitian symmetry of the updated spectrum
"""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.helpers import canon_grid, canon_half, small_scene

PI_REF = 3.141592  # domain.cpp:206-208


def field_only(n=32, L=32.0, chi=2.5, gamma=1.0, M=1.0, T=1.0, v=1.0, phi=None, noise="off", dt=1e-3):
    o = Oracle()
    o.domain([-L / 2] * 3, [L] * 3)
    o.grid_style(n, n, n)
    o.grid_set("phi", phi)
    o.fix_conjugate_volfrac(3, mobility=M, temp=T, volFH=v, gamma=gamma, noise=noise)
    o.fix_floryhuggins(temp=T, volFH=v, chi=chi)
    o.set_dt(dt)
    o.setup()
    return o


@pytest.mark.parametrize("m", [1, 3])
def test_linear_growth_rate(m):
    n, L, phi0, eps = 32, 32.0, 0.5, 1e-7
    chi, gamma, M, T, v, dt = 2.5, 1.0, 1.0, 1.0, 1.0, 1e-3
    x = np.arange(n) * (L / n)
    phi = phi0 + eps * np.cos(2 * math.pi * m * x / L)[None, None, :] * np.ones((n, n, 1))
    o = field_only(n, L, chi, gamma, M, T, v, phi, "off", dt)
    o.run(1)
    out = o.grid_get("phi")
    a1 = (out[0, 0, :] - phi0) @ np.cos(2 * math.pi * m * x / L) * 2 / n
    q = 2 * PI_REF / L * m
    fpp = T / v * (1 / (phi0 * (1 - phi0)) - 2 * chi)
    expect = 1 - M * q * q * dt * (fpp + T / v * gamma * q * q)
    assert abs(a1 / eps - expect) < 1e-6


def test_mass_conserved_to_machine_precision():
    n = 16
    rng = np.random.default_rng(0)
    phi = 0.4 + 0.02 * (rng.random((n, n, n)) - 0.5)
    o = field_only(n, 16.0, phi=phi, noise="reference", dt=1e-4)
    m0 = o.grid_get("phi").sum()
    o.run(20)
    m1 = o.grid_get("phi").sum()
    assert abs(m1 - m0) < 1e-12 * abs(m0)


def test_updated_spectrum_is_hermitian_on_planes():
    n = 16
    rng = np.random.default_rng(1)
    phi = 0.4 + 0.02 * (rng.random((n, n, n)) - 0.5)
    o = field_only(n, 16.0, phi=phi, noise="reference", dt=1e-4)
    o.run(1)
    # after a step the stored ft_phi is the updated (normalised) spectrum
    s = o.grid_get("ft_phi")  # [ky][kz][kx]
    for kx in (0, n // 2):
        p = s[:, :, kx]
        mirror = np.conj(p[(-np.arange(n)) % n][:, (-np.arange(n)) % n])
        real_pts = [(a, b) for a in (0, n // 2) for b in (0, n // 2)]
        mask = np.ones_like(p, bool)
        for a, b in real_pts:
            mask[a, b] = False
        assert np.array_equal(p[mask], mirror[mask])


def test_gridatom_force_vanishes_in_constant_field():
    o = Oracle()
    x, *_ = small_scene(o, phi0=0.4, amp=0.0, with_lj=False)
    o.setup()
    o.stage_gradient()
    o.stage_borders_and_build()
    o.stage_pairs()
    _, _, f, _ = o.atoms_get()
    assert np.abs(f).max() < 1e-12


def test_lj_pair_force_analytic():
    o = Oracle()
    o.domain([0.0] * 3, [16.0] * 3)
    o.grid_style(16, 16, 16)
    o.grid_populate_constant(0.5, 0.0, 1)
    r = 1.05
    x = np.array([[3.0, 3.0, 3.0], [3.0 + r, 3.0, 3.0]])
    o.atoms_create([1, 2], [0, 0], [0, 0], x)
    o.pair_lj_cut(2 ** (1 / 6), 1.0, 1.0)
    o.neighbor(0.3)
    o.setup()
    o.stage_borders_and_build()
    o.stage_pairs()
    _, _, f, _ = o.atoms_get()
    fmag = 48 / r ** 13 - 24 / r ** 7
    assert abs(f[1, 0] - fmag) < 1e-12 * fmag and abs(f[0, 0] + fmag) < 1e-12 * fmag


def brute_half(x, tags, L, lo, cut, zperiodic):
    pairs = set()
    n = len(x)
    for i in range(n):
        for j in range(i + 1, n):
            for sx in (-1, 0, 1):
                for sy in (-1, 0, 1):
                    for sz in ((-1, 0, 1) if zperiodic else (0,)):
                        d = x[i] - (x[j] + np.array([sx, sy, sz]) * L)
                        if d @ d <= cut * cut:
                            code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1)
                            a, b = tags[i], tags[j]
                            pairs.add((a, b, code) if a < b else (b, a, 26 - code))
    return pairs


def brute_grid(x, tags, n, L, lo, cut, zperiodic):
    dx = L / n
    out = set()
    for b in range(len(x)):
        for sx in (-1, 0, 1):
            for sy in (-1, 0, 1):
                for sz in ((-1, 0, 1) if zperiodic else (0,)):
                    p = x[b] + np.array([sx, sy, sz]) * L
                    kmin = np.floor((p - lo - cut) / dx).astype(int)
                    kmax = np.ceil((p - lo + cut) / dx).astype(int)
                    for kz in range(max(kmin[2], 0), min(kmax[2], n - 1) + 1):
                        for ky in range(max(kmin[1], 0), min(kmax[1], n - 1) + 1):
                            for kx in range(max(kmin[0], 0), min(kmax[0], n - 1) + 1):
                                node = np.array([kx * dx + lo, ky * dx + lo, kz * dx + lo])
                                d = node - p
                                if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= cut * cut:
                                    code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1)
                                    out.add(((kz * n + ky) * n + kx, int(tags[b]), code))
    return out


@pytest.mark.parametrize("zghost", ["periodic", "rank1"])
def test_lists_match_brute_force(zghost):
    o = Oracle()
    n, L = 16, 16.0
    x, tags, mol, types = small_scene(o, n=n, L=L, nbeads=120, zghost=zghost)
    o.setup()
    xw, *_ = o.atoms_get()
    cut = 2 ** (1 / 6) + 0.3  # cutneigh = max pair cut + skin (neighbor.cpp:47-55)
    zp = zghost == "periodic"
    assert canon_half(o.half_list()) == brute_half(xw, tags, L, -L / 2, cut, zp)
    assert canon_grid(o.grid_list()) == brute_grid(xw, tags, n, L, -L / 2, cut, zp)

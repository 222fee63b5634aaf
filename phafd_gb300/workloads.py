"""Synthetic workloads of the particle-field step.

Each workload is a seeded, fully synthetic restatement of one benchmark
configuration (no dataset is involved): a periodic cubic box, a grid
initialised by the reference's own `grid_populate constant concentration`
rule (grid.cpp:289-307), semiflexible chains laid down as self-avoiding
random walks of bond length 1.0, and the pair / fix parameters of the
configuration.

`apply(driver, cfg)` issues the same command sequence as a PHAFD input script
(input.cpp:48-299) on any object that exposes the PhafdGPU method names, so
tests drive the GPU library and the CPU oracle identically.
"""
import math

import numpy as np

# Parameters shared by every configuration (WCA beads, gaussian coupling)
_COMMON = dict(
    lj_cut=2.0 ** (1.0 / 6.0), lj_eps=1.0, lj_sigma=1.0,
    ga_style="gaussian", ga_cut=1.0, ga_eps=1.0, ga_width=1.0, ga_phi=0.1,
    gamma=1.0, mobility=1.0, temp=1.0, volFH=1.0, field_temp=0.01,
    bond=1.0, kbond=100.0, bending=10.0, zeta=1.0,
    dt=1e-4, skin=0.3, amp=0.02,
)

CONFIGS = {
    # 64^3, one chain of 200 beads, noise off: the FP64 parity workload
    "64cube_200beads": dict(_COMMON, n=64, L=64.0, origin=-32.0, phi0=0.5, chi=2.5, grid_seed=1,
                            nchains=1, chain_len=200, chain_seed=2, field_noise="off",
                            bead_temp=0.0, steps=1000),
    # 256^3, 64 chains x 500 beads = 32,000 beads, kT = 1: the headline workload
    "256cube_32kbeads": dict(_COMMON, n=256, L=256.0, origin=-128.0, phi0=0.4, chi=3.0, grid_seed=1,
                             nchains=64, chain_len=500, chain_seed=3, field_noise="philox",
                             bead_temp=1.0, steps=5000),
    # 512^3, 2,000 chains x 500 beads = 1,000,000 beads, kT = 1
    "512cube_1Mbeads": dict(_COMMON, n=512, L=512.0, origin=-256.0, phi0=0.45, chi=3.0, grid_seed=1,
                            nchains=2000, chain_len=500, chain_seed=4, field_noise="philox",
                            bead_temp=1.0, steps=10000),
    # small cases for fast tests
    "32cube_64beads": dict(_COMMON, n=32, L=32.0, origin=-16.0, phi0=0.5, chi=2.5, grid_seed=5,
                           nchains=2, chain_len=32, chain_seed=6, field_noise="off",
                           bead_temp=0.0, steps=50),
}


def random_walk_chains(nchains, length, boxlo, L, seed, bond=1.0, min_sep=1.0, max_tries=200):
    """Self-avoiding random walks with exact bond length `bond`.

    Beads of different chains, and non-adjacent beads of one chain, keep at
    least `min_sep` apart (minimum image), so the WCA pair starts finite.
    Positions are unwrapped (chains may leave the box; pbc wraps them).
    Returns x (n,3), tags (1-based, chain-contiguous), mol ids, types (all 0).
    """
    rng = np.random.default_rng(seed)
    cell = max(min_sep, 1e-6)
    ncell = max(1, int(L // cell))
    buckets = {}

    def key(p):
        w = np.floor(((p - boxlo) % L) / (L / ncell)).astype(int) % ncell
        return tuple(w)

    def ok(p, skip):
        k = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    kk = ((k[0] + dx) % ncell, (k[1] + dy) % ncell, (k[2] + dz) % ncell)
                    for idx, q in buckets.get(kk, ()):
                        if idx in skip:
                            continue
                        d = p - q
                        d -= L * np.round(d / L)
                        if d @ d < min_sep * min_sep:
                            return False
        return True

    xs = []
    for c in range(nchains):
        for restart in range(max_tries):
            idx0 = len(xs)
            for attempt in range(max_tries):
                start = boxlo + rng.random(3) * L
                if ok(start, ()):
                    break
            chain = [start]
            buckets.setdefault(key(start), []).append((idx0, start))
            xs.append(start)
            grown = True
            for b in range(1, length):
                prev = chain[-1]
                for attempt in range(max_tries):
                    v = rng.standard_normal(3)
                    v /= np.linalg.norm(v)
                    p = prev + bond * v
                    if ok(p, {len(xs) - 1}):
                        break
                else:
                    grown = False
                    break
                chain.append(p)
                buckets.setdefault(key(p), []).append((len(xs), p))
                xs.append(p)
            if grown:
                break
            # trapped: remove this chain and grow it again from a new start
            for idx in range(idx0, len(xs)):
                kk = key(xs[idx])
                buckets[kk] = [e for e in buckets[kk] if e[0] != idx]
            del xs[idx0:]
        else:
            raise RuntimeError("could not grow a self-avoiding chain")
    x = np.array(xs, dtype=np.float64)
    n = len(x)
    tags = np.arange(1, n + 1, dtype=np.int32)
    mol = np.repeat(np.arange(nchains, dtype=np.int32), length)
    types = np.zeros(n, dtype=np.int32)
    return x, tags, mol, types


def chain_ranges(nchains, length):
    return [(c * length, (c + 1) * length) for c in range(nchains)]


def apply(driver, cfg, chains=None, semiflexible=True, drag=None, zghost="periodic", phi=None):
    """Issue the configuration's script commands on `driver`.  `phi` (a real
    [z][y][x] array) replaces the generated initial field: the state of a
    run continued from host memory."""
    n, L, lo = cfg["n"], cfg["L"], cfg["origin"]
    driver.set_zghost(zghost)
    driver.domain([lo, lo, lo], [L, L, L])
    driver.grid_style(n, n, n)
    if phi is None:
        driver.grid_populate_constant(cfg["phi0"], cfg["amp"], cfg["grid_seed"])
    else:
        driver.grid_set("phi", phi)
    if chains is None:
        chains = random_walk_chains(cfg["nchains"], cfg["chain_len"], lo, L, cfg["chain_seed"], cfg["bond"])
    x, tags, mol, types = chains
    driver.atoms_create(tags, mol, types, x)
    driver.pair_gridatom(cfg["ga_style"], cfg["ga_cut"])
    driver.pair_gridatom_coeff(0, epsilon=cfg["ga_eps"], nucwidth=cfg["ga_width"], phi=cfg["ga_phi"])
    driver.pair_lj_cut(cfg["lj_cut"], cfg["lj_eps"], cfg["lj_sigma"])
    driver.neighbor(cfg["skin"])
    ranges = chain_ranges(cfg["nchains"], cfg["chain_len"])
    if semiflexible:
        driver.fix_semiflexible(ranges, bondlength=cfg["bond"], zeta_para=cfg["zeta"], zeta_perp=cfg["zeta"],
                                bending=cfg["bending"], temp=cfg["bead_temp"], kbond=cfg["kbond"],
                                seed=cfg["chain_seed"] + 100, noise="philox" if cfg["bead_temp"] > 0 else "off")
    if drag is not None:
        driver.fix_drag(ranges, drag)
    # The conjugate fix's temp sets both the conserved-noise amplitude and the
    # gradient coefficient kappa = temp/volFH*gamma (conjugate_volfrac.cpp:80-108).
    # The noise runs at field_temp while gamma is rescaled so that kappa keeps
    # its value temp/volFH*gamma: at field temp 1 on a unit-spacing grid the
    # explicit update is driven through the Flory-Huggins log singularity
    # within a few dozen steps of dt = 1e-4.
    driver.fix_conjugate_volfrac(cfg["grid_seed"] + 10, mobility=cfg["mobility"], temp=cfg["field_temp"],
                                 volFH=cfg["volFH"], gamma=cfg["gamma"] * cfg["temp"] / cfg["field_temp"],
                                 noise=cfg["field_noise"])
    driver.fix_floryhuggins(temp=cfg["temp"], volFH=cfg["volFH"], chi=cfg["chi"])
    driver.set_dt(cfg["dt"])
    return chains


def algorithmic_bytes_per_step(cfg, s):
    """B_step = 6 s N + 10 s N_c + N_b (5 s P + 24 s): one compulsory read and
    write per 3D FFT with the pointwise stages fused, plus the bead terms
    (P = 4.19 grid nodes within the coupling width 1)."""
    n = cfg["n"]
    N = n ** 3
    Nc = (n // 2 + 1) * n * n
    Nb = cfg["nchains"] * cfg["chain_len"]
    P = 4.19
    return 6 * s * N + 10 * s * Nc + Nb * (5 * s * P + 24 * s)


def nbeads(cfg):
    return cfg["nchains"] * cfg["chain_len"]


__all__ = ["CONFIGS", "random_walk_chains", "chain_ranges", "apply", "algorithmic_bytes_per_step", "nbeads"]


def _selfcheck():  # pragma: no cover - quick manual check
    x, *_ = random_walk_chains(1, 50, -8.0, 16.0, 1)
    d = np.linalg.norm(np.diff(x, axis=0), axis=1)
    assert np.allclose(d, 1.0)
    return math.isfinite(float(x.sum()))

"""Shared helpers of the test suite."""
import numpy as np


def canon_half(rows):
    """Canonical set of unordered bead pairs: (min tag, max tag, image code of
    the larger tag relative to the smaller)."""
    out = set()
    for a, b, code in np.asarray(rows).tolist():
        if a < b:
            out.add((a, b, code))
        else:
            out.add((b, a, 26 - code))
    return out


def canon_grid(rows):
    return set(tuple(r) for r in np.asarray(rows).tolist())


def rel_err(a, b):
    a = np.asarray(a); b = np.asarray(b)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)


def small_scene(driver, n=32, L=32.0, nbeads=64, seed=7, zghost="periodic", style="gaussian",
                phi0=0.5, amp=0.2, with_lj=True, cut=1.0, skin=0.3, chain=False):
    """A small box with random beads near every face (so images matter)."""
    rng = np.random.default_rng(seed)
    lo = -L / 2
    driver.set_zghost(zghost)
    driver.domain([lo] * 3, [L] * 3)
    driver.grid_style(n, n, n)
    driver.grid_populate_constant(phi0, amp, seed)
    if chain:
        from phafd_gb300.workloads import random_walk_chains
        x, tags, mol, types = random_walk_chains(2, nbeads // 2, lo, L, seed)
    else:
        x = lo + rng.random((nbeads, 3)) * L
        # put a few beads close to faces and corners
        x[:8] = lo + np.array([[0.2, 5, 5], [L - 0.3, 6, 5], [5, 0.1, 7], [5, L - 0.2, 7],
                               [9, 9, 0.3], [9, 9, L - 0.4], [0.2, 0.3, 0.4], [L - 0.1, L - 0.2, L - 0.3]])
        tags = np.arange(1, nbeads + 1, dtype=np.int32)
        mol = np.zeros(nbeads, np.int32)
        types = (np.arange(nbeads) % 2).astype(np.int32)
    driver.atoms_create(tags, mol, types, x)
    if style is not None:
        driver.pair_gridatom(style, cut)
        driver.pair_gridatom_coeff(0, epsilon=1.0, nucwidth=cut, phi=0.1)
        if types.max() > 0:
            driver.pair_gridatom_coeff(1, epsilon=-0.5, nucwidth=0.8 * cut, phi=0.3)
    if with_lj:
        driver.pair_lj_cut(2 ** (1 / 6), 1.0, 1.0)
    driver.neighbor(skin)
    return x, tags, mol, types


def shell_sk(phi, nbins=None):
    """Shell-averaged structure factor of a real cubic field [z][y][x]: |F(k)|^2
    of the r2c spectrum summed over integer shells floor(|n|) of the
    wavenumber index (the k = 0 mode left out; modes with 0 < kx < N/2 count
    twice, for their mirror), divided by the shell's mode count."""
    phi = np.asarray(phi, np.float64)
    n = phi.shape[0]
    F = np.fft.rfftn(phi)
    p = np.abs(F) ** 2
    kz = np.fft.fftfreq(n) * n
    ky = np.fft.fftfreq(n) * n
    kx = np.arange(n // 2 + 1, dtype=np.float64)
    r = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    b = np.floor(r + 1e-9).astype(np.int64)
    w = np.where((kx == 0) | (kx == n // 2), 1.0, 2.0)[None, None, :] * np.ones_like(p)
    w[0, 0, 0] = 0.0
    nb = nbins or n // 2
    keep = b < nb
    s = np.bincount(b[keep], (w * p)[keep], minlength=nb)
    c = np.bincount(b[keep], w[keep], minlength=nb)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(c > 0, s / np.maximum(c, 1), 0.0)


def sk_rel_err(a, b):
    """max over shells (k >= 1) of |S_a - S_b| / S_b."""
    sa, sb = shell_sk(a), shell_sk(b)
    m = sb[1:] > 0
    return float(np.max(np.abs(sa[1:][m] - sb[1:][m]) / sb[1:][m]))

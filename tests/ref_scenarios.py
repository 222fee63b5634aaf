"""Parity scenarios pinned by the reference's own code.

Each scenario is a reference input script (its syntax, input.cpp:48-299)
plus the equivalent command sequence on any driver with the PhafdGPU method
names (the oracle, the GPU library).  tests/golden/make_ref_golden.py runs
the scripts through the reference's sources compiled against stand-ins of
their absent third-party libraries (oracle/refpin) and stores the final
states as fixtures; the tests replay the same commands on the oracle (CPU)
and on the FP64 GPU path and compare.

The reference runs on one MPI rank, so the replays use its one-rank z-ghost
semantics (no periodic z images of beads, comm_brick.cpp:300-318) and its
mt19937 field noise (the conjugate fix's draw order, conjugate.cpp:163-247).
Beads move with fix atom/drag: the chain integrator of fix
atom/semiflexible (the external beadrodpmer library) is not available.
"""
import numpy as np

from phafd_gb300 import workloads as W

_BASE = dict(
    boxlo=(-8.0, -8.0, -8.0), period=(16.0, 16.0, 16.0), grid=(16, 16, 16), phi0=0.5, var=0.2, grid_seed=5,
    nbeads=80, bead_seed=7, style="gaussian", cut=1.0, coeffs=((0, 1.0, 1.0, 0.1), (1, -0.5, 0.8, 0.3)),
    lj=True, skin=0.3, drag=1.0, conj=(15, 1.0, 0.01, 1.0, 100.0), fh=(1.0, 1.0, 2.5), gradphi=None,
    dt=1e-3, steps=20, compute_pair=False, min_sep=1.0,
)

SCENARIOS = {
    # gaussian coupling, lj/cut, drag, conjugate noise, Flory-Huggins
    "gaussian_drag": dict(_BASE),
    # the LJish coupling (pair_gridatom_lj_ish.cpp)
    "ljish_drag": dict(_BASE, style="LJish", coeffs=((0, 1.0, 1.0, 0.1), (1, 0.5, 0.9, 0.6))),
    # the linear LJish coupling (pair_gridatom_lj_ish_linear.cpp), with the
    # per-bead forces of that style through compute pair at dump steps
    "ljish_linear_pair": dict(_BASE, style="LJish/linear", coeffs=((0, -1.0, 1.0, None), (1, 2.0, 0.9, None)),
                              compute_pair=True, steps=12),
    # anisotropic box and grid: the y/z swap of dq (domain.cpp:206-208)
    "aniso_box": dict(_BASE, boxlo=(-8.0, -12.0, -16.0), period=(16.0, 24.0, 32.0), grid=(16, 16, 32), nbeads=120,
                      steps=15),
    # a field far outside [0, 1]: the Flory-Huggins reflections and their
    # counters, and fix grid/gradphi every step; no beads
    "field_reflections": dict(_BASE, nbeads=0, var=1.6, fh=(1.0, 1.0, 3.0), gradphi="every", steps=8),
    # beads placed inside each other's repulsive range and a strong drag:
    # fast beads, neighbor rebuilds
    "rebuilds": dict(_BASE, nbeads=100, steps=40, drag=5.0, min_sep=0.93),
}


def bead_inputs(sc):
    """Beads at least min_sep apart (minimum image), alternating types 0 and
    1, all in molecule 0: (tags, mol, types, x)."""
    n = sc["nbeads"]
    if n == 0:
        return (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 3)))
    lo = sc["boxlo"][0]
    L = min(sc["period"])
    x, tags, _, _ = W.random_walk_chains(n, 1, lo, L, sc["bead_seed"], 1.0, min_sep=sc["min_sep"])
    for d in range(3):  # spread over the full (possibly longer) axes
        x[:, d] = sc["boxlo"][d] + (x[:, d] - lo) % L * (sc["period"][d] / L)
    types = (np.arange(n) % 2).astype(np.int32)
    return tags.astype(np.int32), np.zeros(n, np.int32), types, x


def atoms_file_text(beads):
    tags, mol, types, x = beads
    return "".join("%d %d %d %.17g %.17g %.17g\n" % (tags[i], mol[i], types[i], *x[i]) for i in range(len(tags)))


def script(sc, atoms_path, dump_dir=None):
    """The scenario as a reference input script."""
    lo, L, g = sc["boxlo"], sc["period"], sc["grid"]
    lines = [
        "domain boxdims %r %r %r boxorigin %r %r %r" % (L[0], L[1], L[2], lo[0], lo[1], lo[2]),
        "grid_style %d %d %d concentration" % g,
        "grid_populate constant concentration %r %r %d" % (sc["phi0"], sc["var"], sc["grid_seed"]),
        "atom_style polymer natoms %d" % sc["nbeads"],
        "atom_populate read_atoms %s" % atoms_path,
    ]
    if sc["nbeads"]:
        lines.append("pair gridatom/%s %r" % (sc["style"], sc["cut"]))
        for t, eps, width, phi in sc["coeffs"]:  # the linear style takes no phi
            lines.append("pairCoeffs %d epsilon %r nucwidth %r" % (t, eps, width) + (" phi %r" % phi if phi is not None else ""))
        if sc["lj"]:
            lines.append("pair lj/cut 1.122462048309373 1.0 1.0")
        lines.append("neighbor %r" % sc["skin"])
        lines.append("group beads atom <> 1 %d" % sc["nbeads"])
        lines.append("fix atom/drag drg beads %r" % sc["drag"])
    else:  # the communication set-up still needs a cutoff (the reference faults without one)
        lines.append("neighbor %r" % sc["skin"])
    if sc["gradphi"]:
        lines.append("fix grid/gradphi gradphi %s" % sc["gradphi"])
    seed, mob, temp, vol, gamma = sc["conj"]
    lines.append("fix grid/conjugate/volfrac volfrac %d mobility %r temp %r volFH %r gamma %r"
                 % (seed, mob, temp, vol, gamma))
    t, v, chi = sc["fh"]
    lines.append("fix grid/floryhuggins chempot temp %r chi %r volFH %r" % (t, chi, v))
    if sc["compute_pair"]:
        lines.append("compute pair cpair gridatom/%s" % sc["style"])
        lines.append("dump beads atom/owned %s/beads 4 attributes 3 x ID c_cpair" % dump_dir)
    lines += ["timestep 0", "dt %r" % sc["dt"], "run %d" % sc["steps"]]
    return "\n".join(lines) + "\n"


def apply(driver, sc, beads):
    """The scenario's commands on a driver with the PhafdGPU method names
    (one-rank z ghosts, the reference's mt19937 field noise)."""
    driver.set_zghost("rank1")
    driver.domain(list(sc["boxlo"]), list(sc["period"]))
    driver.grid_style(*sc["grid"])
    driver.grid_populate_constant(sc["phi0"], sc["var"], sc["grid_seed"])
    tags, mol, types, x = beads
    if sc["nbeads"]:
        driver.atoms_create(tags, mol, types, x)
        driver.pair_gridatom(sc["style"], sc["cut"])
        for t, eps, width, phi in sc["coeffs"]:
            driver.pair_gridatom_coeff(t, epsilon=eps, nucwidth=width, phi=phi)
        if sc["lj"]:
            driver.pair_lj_cut(1.122462048309373, 1.0, 1.0)
        driver.neighbor(sc["skin"])
        driver.fix_drag([(0, sc["nbeads"])], sc["drag"])
    if sc["gradphi"]:
        driver.fix_gradphi(once=sc["gradphi"] == "once")
    seed, mob, temp, vol, gamma = sc["conj"]
    driver.fix_conjugate_volfrac(seed, mobility=mob, temp=temp, volFH=vol, gamma=gamma, noise="reference")
    t, v, chi = sc["fh"]
    driver.fix_floryhuggins(temp=t, volFH=v, chi=chi)
    driver.set_dt(sc["dt"])
    driver.set_timestep(0)


def shift_codes(x_all, tags_all, nowned, period, js):
    """Image code (sx+1) + 3 (sy+1) + 9 (sz+1) of copy j relative to the owned
    bead with the same tag."""
    own = {int(t): i for i, t in enumerate(tags_all[:nowned])}
    out = []
    for j in js:
        o = own[int(tags_all[j])]
        code, mul = 0, 1
        for d in range(3):
            s = int(np.rint((x_all[j, d] - x_all[o, d]) / period[d]))
            code += (s + 1) * mul
            mul *= 3
        out.append(code)
    return np.asarray(out, np.int32)

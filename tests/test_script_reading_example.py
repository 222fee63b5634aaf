"""The reference's example script (examples/test/reading.in) on phafd_gpu.

The script below keeps that example's commands in its order: a polymer
atom style read from a file, pair gridatom/LJish/linear with two pairCoeffs
lines, pair lj/cut, neighbor, group, fix atom/semiflexible/notether, fix
grid/conjugate/volfrac, fix grid/floryhuggins, compute pair on the coupling
style, an atom dump with c_droppolyforces and a grid dump with phi, chempot
and gradphi_x/y/z.  Sizes are small (32^3 grid, two 32-bead chains) and the
run is a plain run of 20 steps (the example ends with run_until_touching,
whose dumps this interpreter refuses).

CPU: the script parses (dry run).  GPU (FP64): the dumps of steps 10 and 20
hold what the oracle has after the same commands: phi, chempot (which the
compute's re-run of the pair adds its deposit to, as the reference's does),
the gradient of the step's starting phi, and compute pair's per-bead forces
of the coupling style.
"""
import os
import subprocess

import numpy as np
import pytest

from phafd_gb300 import workloads as W
from tests.helpers import rel_err

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "phafd_gb300", "_build", "phafd_gpu")

SCRIPT = """# set global parameters
package gpu precision 64

domain boxdims 32.0 32.0 32.0 boxorigin -16.0 -16.0 -16.0

grid_style 32 32 32 concentration

grid_populate constant concentration ${phi0} ${phi_var} ${seed1}
atom_style polymer natoms ${Nbeads}
atom_populate read_atoms polymercoords/run${run}_empty_p%.data

pair gridatom/LJish/linear ${bondlength}
pairCoeffs 0 epsilon ${attract} nucwidth ${bondlength}
pairCoeffs 1 epsilon ${repel} nucwidth ${bondlength}

pair lj/cut ${ljcut} ${ljeps} ${ljsigma}

neighbor ${nskin}

group nt_pmers molecule 0 1

fix atom/semiflexible/notether nt_pmers nt_pmers ${seed2} bondlength ${bondlength} zeta_para ${zeta_para} zeta_perp ${zeta_perp} bending ${bending} temp ${temp}

fix grid/conjugate/volfrac volfrac ${seed3} mobility ${mobility} temp ${temp} volFH ${v0} gamma ${gamma}

fix grid/floryhuggins chempot temp ${temp} chi ${chi} volFH ${v0}

compute pair droppolyforces gridatom/LJish/linear

dump atoms atom/owned vtkfiles/run${run}atom 10 attributes 8 x ux ix F c_droppolyforces ID molID type decimalplaces 15 fmt e

dump realgrid grid vtkfiles/run${run}field 10 attributes 5 phi chempot gradphi_x gradphi_y gradphi_z

timestep 0
dt ${dt}

run 20
"""

VARS = dict(phi0="0.5", phi_var="0.02", seed1="5", Nbeads="64", run="0", bondlength="1.0", attract="-1.0",
            repel="0.5", ljcut="1.122462048309373", ljeps="1.0", ljsigma="1.0", nskin="0.3", seed2="106",
            zeta_para="1.0", zeta_perp="1.0", bending="10.0", temp="0.01", seed3="15", mobility="1.0", v0="1.0",
            gamma="100.0", chi="2.5", dt="5e-4")


@pytest.fixture(scope="module")
def exe():
    from phafd_gb300 import build as B
    B.build()
    return EXE


def scene(tmp_path):
    cfg = W.CONFIGS["32cube_64beads"]
    x, tags, mol, types = W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"],
                                               cfg["chain_seed"])
    types = (np.arange(len(tags)) % 2).astype(np.int32)  # both coefficient lines in use
    (tmp_path / "polymercoords").mkdir()
    with open(tmp_path / "polymercoords" / "run0_empty_p0.data", "w") as f:
        for i in range(len(x)):
            f.write("%d %d %d %.17g %.17g %.17g\n" % (tags[i], mol[i], types[i], *x[i]))
    (tmp_path / "vtkfiles").mkdir()
    (tmp_path / "in.reading").write_text(SCRIPT)
    return x, tags, mol, types


def run(exe, tmp_path, *extra):
    args = [exe, "-in", "in.reading", "-sf", "gpu"]
    for k, v in VARS.items():
        args += ["-var", k, v]
    return subprocess.run(args + list(extra), cwd=tmp_path, capture_output=True, text=True, timeout=600)


def test_reading_example_parses(exe, tmp_path):
    scene(tmp_path)
    r = run(exe, tmp_path, "-dry-run")
    assert r.returncode == 0, r.stderr
    assert r.stderr == ""


def vti_arrays(path, n, names):
    raw = open(path, "rb").read()
    at = raw.index(b"\n_") + 2
    out = {}
    for name in names:
        assert int.from_bytes(raw[at:at + 4], "little") == 8 * n
        out[name] = np.frombuffer(raw, "<f8", n, at + 4)
        at += 4 + 8 * n
    return out


def vtp_array(text, name):
    head = '<DataArray Name="%s" type="Float64" NumberOfComponents="3" format="ascii">\n' % name
    return np.array(text.split(head)[1].split("\n")[0].split(), np.float64).reshape(-1, 3)


@pytest.mark.gpu
def test_reading_example_dumps_match_oracle(exe, tmp_path, gpu_lib):
    from oracle.oracle import Oracle
    x, tags, mol, types = scene(tmp_path)
    r = run(exe, tmp_path)
    assert r.returncode == 0, r.stderr
    v = {k: float(val) if k not in ("seed1", "seed2", "seed3", "Nbeads", "run") else int(val)
         for k, val in VARS.items()}
    o = Oracle()
    o.domain([-16.0] * 3, [32.0] * 3)
    o.grid_style(32, 32, 32)
    o.grid_populate_constant(v["phi0"], v["phi_var"], v["seed1"])
    o.atoms_create(tags, mol, types, x)
    o.pair_gridatom("LJish/linear", v["bondlength"])
    o.pair_gridatom_coeff(0, epsilon=v["attract"], nucwidth=v["bondlength"])
    o.pair_gridatom_coeff(1, epsilon=v["repel"], nucwidth=v["bondlength"])
    o.pair_lj_cut(v["ljcut"], v["ljeps"], v["ljsigma"])
    o.neighbor(v["nskin"])
    o.fix_semiflexible([(0, 32), (32, 64)], bondlength=v["bondlength"], zeta_para=v["zeta_para"],
                       zeta_perp=v["zeta_perp"], bending=v["bending"], temp=v["temp"], kbond=100.0,
                       seed=v["seed2"], noise="philox")
    o.fix_conjugate_volfrac(v["seed3"], mobility=v["mobility"], temp=v["temp"], volFH=v["v0"], gamma=v["gamma"],
                            noise="philox")
    o.fix_floryhuggins(temp=v["temp"], volFH=v["v0"], chi=v["chi"])
    o.set_dt(v["dt"])
    o.set_timestep(0)
    o.setup()
    n = 32 ** 3
    for step in (10, 20):
        o.run(10)
        forces = o.compute_pair("gridatom")  # also leaves its deposit in chempot
        grid = vti_arrays(tmp_path / "vtkfiles" / ("run0field_p0_%d.vti" % step), n,
                          ("phi", "chempot", "gradphi_x", "gradphi_y", "gradphi_z"))
        assert rel_err(grid["phi"], o.grid_get("phi").ravel()) < 1e-10
        assert rel_err(grid["chempot"], o.grid_get("chempot").ravel()) < 1e-10
        for a, f in (("gradphi_x", "gradx"), ("gradphi_y", "grady"), ("gradphi_z", "gradz")):
            assert rel_err(grid[a], o.grid_get(f).ravel()) < 1e-10, a
        vtp = (tmp_path / "vtkfiles" / ("run0atom_p0_%d.vtp" % step)).read_text()
        assert np.abs(forces).max() > 0
        assert rel_err(vtp_array(vtp, "c_droppolyforces"), forces) < 1e-10
        assert rel_err(vtp_array(vtp, "F"), o.atoms_get()[2]) < 1e-9

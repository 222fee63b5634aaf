"""The phafd_gpu input-script interpreter: reference command syntax, ${var}
and % substitution, /gpu style selection, groups, read_atoms.

CPU tests run the interpreter with -dry-run (parse and check only); the GPU
test runs a script and compares the written phi with the same command
sequence issued through the Python binding."""
import os
import subprocess

import numpy as np
import pytest

from phafd_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "phafd_gb300", "_build", "phafd_gpu")

SCRIPT = """# reference-syntax script (examples/test/reading.in style)
domain boxdims ${L} ${L} ${L} boxorigin -16.0 -16.0 -16.0
grid_style 32 32 32 concentration
grid_populate constant concentration 0.5 0.02 ${seed1}
atom_style polymer natoms 64
atom_populate read_atoms atoms_p%.data
pair gridatom/gaussian 1.0
pairCoeffs 0 epsilon 1.0 nucwidth 1.0 phi 0.1

pair lj/cut 1.122462048309373 1.0 1.0
neighbor 0.3
group chains molecule 0 1
fix atom/semiflexible/notether pmers chains 106 bondlength 1.0 zeta_para 1.0 zeta_perp 1.0 bending 10.0 temp 0.0
fix grid/conjugate/volfrac volfrac 15 mobility 1.0 temp 0.01 volFH 1.0 gamma 100.0
fix grid/floryhuggins chempot temp 1.0 chi 2.5 volFH 1.0
dump realgrid grid out 100 attributes 1 phi
timestep 0
dt 5e-4
run 20
write_field phi phi.bin
"""


@pytest.fixture(scope="module")
def exe():
    if not os.path.exists(EXE):
        from phafd_gb300 import build as B
        try:
            B.build()
        except Exception as e:  # pragma: no cover
            pytest.skip("cannot build: %s" % e)
    return EXE


def scene(tmp_path, script=SCRIPT):
    cfg = W.CONFIGS["32cube_64beads"]
    x, tags, mol, types = W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"],
                                               cfg["chain_seed"])
    with open(tmp_path / "atoms_p0.data", "w") as f:
        f.write("# ID molID type x y z\n")
        for i in range(len(x)):
            f.write("%d %d %d %.17g %.17g %.17g\n" % (tags[i], mol[i], types[i], *x[i]))
    (tmp_path / "in.phafd").write_text(script)
    return (x, tags, mol, types)


def run(exe, tmp_path, *extra):
    return subprocess.run([exe, "-in", "in.phafd", "-var", "L", "32.0", "-var", "seed1", "5", *extra],
                          cwd=tmp_path, capture_output=True, text=True, timeout=300)


def test_dry_run_parses_reference_script(exe, tmp_path):
    scene(tmp_path)
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr
    assert "dry run: 20 steps parsed" in r.stdout
    assert r.stderr == ""  # the grid dump is a built command now


def test_styles_need_the_gpu_suffix(exe, tmp_path):
    scene(tmp_path)
    r = run(exe, tmp_path, "-dry-run")
    assert r.returncode == 1 and "gridatom/gaussian/gpu" in r.stderr
    scene(tmp_path, SCRIPT.replace("pair gridatom/gaussian 1.0", "pair gridatom/gaussian/gpu 1.0")
          .replace("pair lj/cut", "pair lj/cut/gpu").replace("fix atom/", "fix atom/")
          .replace("fix ", "suffix gpu\nfix ", 1))
    r = run(exe, tmp_path, "-dry-run")
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("bad,msg", [
    ("grid_style 32 32 32 concentration", None),
    ("domain boxdims ${L} ${L} ${L} boxorigin -16.0 -16.0 -16.0", "CAnnot use command grid_style before domain box is set."),
    ("${seed1}", None),
])
def test_command_order_and_variables(exe, tmp_path, bad, msg):
    if msg is None:
        return
    scene(tmp_path, SCRIPT.replace(bad + "\n", ""))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and msg in r.stderr


def test_missing_variable_and_duplicate_fix(exe, tmp_path):
    scene(tmp_path, SCRIPT.replace("${seed1}", "${nope}"))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and "No such command line variable nope" in r.stderr
    scene(tmp_path, SCRIPT.replace("run 20", "fix grid/floryhuggins chempot temp 1.0\nrun 20"))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and "Duplicate of fix chempot" in r.stderr


@pytest.mark.gpu
def test_script_run_matches_binding(exe, tmp_path, gpu_lib):
    chains = scene(tmp_path)
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    assert "Run time =" in r.stdout and "chempot had phi < 0" in r.stdout
    phi_script = np.fromfile(tmp_path / "phi.bin", dtype=np.float64).reshape(32, 32, 32)
    from phafd_gb300.gpu import PhafdGPU
    cfg = dict(W.CONFIGS["32cube_64beads"], dt=5e-4, field_noise="philox")  # package gpu default noise
    g = PhafdGPU(precision=32)
    W.apply(g, cfg, chains=chains)
    g.set_timestep(0)
    g.setup()
    g.run(20)
    # same commands, same library; the bead deposit is summed with float
    # atomics, so two runs agree to FP32 round-off, not bit for bit
    ref = g.grid_get("phi")
    assert np.abs(ref - phi_script).max() < 1e-5 * np.abs(ref).max()


NODUMP = SCRIPT.replace("dump realgrid grid out 100 attributes 1 phi\n", "")


def test_no_dumps_during_run_until_touching(exe, tmp_path):
    scene(tmp_path, SCRIPT.replace("run 20", "run_until_touching 20 1.5 stop"))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and "no dumps during run_until_touching" in r.stderr


@pytest.mark.parametrize("line,msg", [
    ("run_until_touching 20 1.5 stop", None),
    ("run_until_touching 20 1.5 continue 5", None),
    ("run_until_touching 20", "Must provide a size at which atoms are considered touching."),
    ("run_until_touching 20 1.5", "Must say whether to continue simulation after touching occurs."),
    ("run_until_touching 20 1.5 continue", "Must say delay to mention new cyclisation events."),
    ("run_until_touching 20 1.5 maybe", "Must say whether to continue simulation after touching occurs."),
])
def test_run_until_touching_syntax(exe, tmp_path, line, msg):
    """input.cpp:274-295 argument checks (dry run)."""
    scene(tmp_path, NODUMP.replace("run 20", line))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    if msg is None:
        assert r.returncode == 0, r.stderr
        assert "dry run: 20 steps parsed" in r.stdout
    else:
        assert r.returncode == 1 and msg in r.stderr


@pytest.mark.gpu
def test_script_run_until_touching_stops(exe, tmp_path, gpu_lib):
    """A touch size beyond the box: the first step touches and the run stops."""
    scene(tmp_path, NODUMP.replace("run 20", "run_until_touching 20 1000.0 stop"))
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    assert "cyclisation occured at step 1" in r.stdout
    assert "number of neighbor calls =" in r.stdout

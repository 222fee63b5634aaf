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
    from phafd_gb300 import build as B
    try:
        B.build()  # incremental: relinks the host program when a source or header changed
    except Exception as e:  # pragma: no cover
        if not os.path.exists(EXE):
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


DUMPS = SCRIPT.replace("dump realgrid grid out 100 attributes 1 phi\n",
                       "compute grid/cluster cl phi 0.5 gt\n"
                       "dump beads atom/owned vtk/beads 10 attributes 3 x ID type decimalplaces 12 fmt e\n"
                       "dump fields grid vtk/fields 10 attributes 3 phi chempot c_cl\n"
                       "dump traj lammpsatom vtk/traj 10 attributes 2 ID x\n")


def test_dump_commands_parse(exe, tmp_path):
    scene(tmp_path, DUMPS)
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr
    assert r.stderr == ""
    for bad, msg in [("attributes 3 phi chempot c_cl", "attributes 3 phi chempot c_nope"),
                     ("attributes 3 x ID type", "attributes 3 x ID bogus")]:
        scene(tmp_path, DUMPS.replace(bad, msg))
        r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
        assert r.returncode == 1


@pytest.mark.gpu
def test_script_dumps_match_fields(exe, tmp_path, gpu_lib):
    """Atom, grid (phi, chempot, cluster labels) and LAMMPS-style dumps on
    steps 0, 10 and 20 of a script run: the last grid dump holds the phi the
    script writes after the run, its labels equal an independent periodic
    labelling of that phi, and the bead positions agree with a binding run."""
    from tests.cluster_ref import periodic_min_id_labels
    chains = scene(tmp_path, DUMPS)
    (tmp_path / "vtk").mkdir()
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    for t in (0, 10, 20):
        assert "Saving on step %d" % t in r.stdout
        for name in ("beads_p0_%d.vtp", "beads_%d.pvtp", "fields_p0_%d.vti", "fields_%d.pvti"):
            assert (tmp_path / "vtk" / (name % t)).exists(), name % t
    pvd = (tmp_path / "vtk" / "fields.pvd").read_text()
    assert pvd.count("<DataSet ") == 3 and pvd.endswith("</Collection>\n</VTKFile>")
    raw = (tmp_path / "vtk" / "fields_p0_20.vti").read_bytes()
    at = raw.index(b"\n_") + 2
    n = 32 ** 3
    arrays = []
    for c in range(3):
        assert int.from_bytes(raw[at:at + 4], "little") == 8 * n
        arrays.append(np.frombuffer(raw, "<f8", n, at + 4).reshape(32, 32, 32))
        at += 4 + 8 * n
    phi = np.fromfile(tmp_path / "phi.bin", dtype=np.float64).reshape(32, 32, 32)
    assert np.array_equal(arrays[0], phi)
    assert np.isfinite(arrays[1]).all() and np.abs(arrays[1]).max() > 0
    want, _ = periodic_min_id_labels(phi, 0.5, True)
    assert np.array_equal(arrays[2].astype(np.int64), want.astype(np.int64))
    vtp = (tmp_path / "vtk" / "beads_p0_20.vtp").read_text()
    body = vtp.split('format="ascii">\n')[1].split("\n</DataArray>")[0]
    x = np.array(body.split(), dtype=np.float64).reshape(-1, 3)
    from phafd_gb300.gpu import PhafdGPU
    cfg = dict(W.CONFIGS["32cube_64beads"], dt=5e-4, field_noise="philox")
    g = PhafdGPU(precision=32)
    W.apply(g, cfg, chains=chains)
    g.set_timestep(0)
    g.setup()
    g.run(20)
    xb = g.atoms_get()[0]
    assert x.shape == xb.shape
    assert np.abs(x - xb).max() < 1e-5 * np.abs(xb).max()
    lmp = (tmp_path / "vtk" / "traj_p0.lmmpstrj").read_text()
    assert lmp.count("ITEM: TIMESTEP") == 3 and "ITEM: ATOMS ID x y z \n" in lmp


def vtp_array(text, name):
    """the values of one ascii DataArray of a .vtp file"""
    head = '<DataArray Name="%s" type="Float64" NumberOfComponents="3" format="ascii">\n' % name
    return np.array(text.split(head)[1].split("\n")[0].split(), np.float64).reshape(-1, 3)


def restart_files(tmp_path, attrs_grid=("phi",), attrs_atoms=("x", "ID", "type", "molID", "ix"), nz=32):
    """A step-10 .vti / .vtp pair in the dump writer's format (restated in
    tests/test_vtk_dump.py) for the 32^3 grid and 64 beads of SCRIPT."""
    from tests.test_vtk_dump import expect_vti, expect_vtp
    cfg = W.CONFIGS["32cube_64beads"]
    x, tags, mol, types = W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"],
                                               cfg["chain_seed"])
    rng = np.random.default_rng(3)
    g = dict(nx=32, ny=32, nz=nz, origin=(-16.0,) * 3, spacing=(1.0,) * 3,
             fields={a: 0.5 + 0.02 * rng.standard_normal(32 * 32 * nz) for a in attrs_grid})
    (tmp_path / "rs").mkdir(exist_ok=True)
    (tmp_path / "rs" / "g_p0_10.vti").write_bytes(expect_vti(g, list(attrs_grid)))
    n = len(tags)
    img = (512 << 20) | (512 << 10) | 512
    a = dict(n=n, x=np.asarray(x).reshape(-1), ux=np.asarray(x).reshape(-1), F=np.zeros(3 * n),
             ints=dict(ID=tags, type=types, molID=mol, ix=np.full(n, img), label=np.zeros(n, int)))
    (tmp_path / "rs" / "b_p0_10.vtp").write_text(expect_vtp(a, list(attrs_atoms), 16, "e"))


RESTART = (SCRIPT.replace("grid_populate constant concentration 0.5 0.02 ${seed1}",
                          "grid_populate read_dump rs/g_p0_10.vti attributes 1 phi")
           .replace("atom_populate read_atoms atoms_p%.data",
                    "atom_populate read_dump rs/b_p%_10.vtp attributes 5 x ID type molID ix")
           .replace("timestep 0", "timestep 10").replace("run 20", "run 10"))


def test_restart_commands_parse(exe, tmp_path):
    scene(tmp_path, RESTART)
    restart_files(tmp_path)
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("edit,files,msg", [
    (("attributes 1 phi", "attributes 1 chempot"), {}, "Read dump needs attribute phi."),
    (("attributes 1 phi", "attributes 2 phi chempot"), {}, "Not all attributes requested in read_dump command"),
    (None, {"nz": 31}, "incorrect size phi in file."),
    (("rs/g_p0_10.vti", "rs/none.vti"), {}, "file not found."),
    (("attributes 5 x ID type molID ix", "attributes 4 x ID type molID"), {}, "Read dump needs attribute ix."),
    (("attributes 5 x ID type molID ix", "attributes 6 x ID type molID ix F"), {}, "Only found attributes"),
    (("attributes 1 phi", "attributes 1 c_cl"), {}, "Cannot read computes from dump"),
])
def test_restart_errors(exe, tmp_path, edit, files, msg):
    """read_dump.cpp error checks, raised by the dry run."""
    scene(tmp_path, RESTART.replace(*edit) if edit else RESTART)
    restart_files(tmp_path, **files)
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and msg in r.stderr, r.stderr


@pytest.mark.gpu
def test_restart_continues_the_run(exe, tmp_path, gpu_lib):
    """Run 20 steps with dumps on step 10; restart a second script from the
    step-10 files (grid_populate / atom_populate read_dump, timestep 10) and
    run 10 steps: both end on the same phi and bead positions.  The noise is
    keyed by (seed, step), so only the summation order of the rebuilt
    neighbor lists and of the FP64 deposit atomics differs."""
    dumps = ("package gpu precision 64\n" + SCRIPT).replace(
        "dump realgrid grid out 100 attributes 1 phi\n",
        "dump beads atom/owned rs/b 10 attributes 6 x ID type molID ix ux decimalplaces 16 fmt e\n"
        "dump fields grid rs/g 10 attributes 1 phi\n")
    scene(tmp_path, dumps)
    (tmp_path / "rs").mkdir()
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    phi_a = np.fromfile(tmp_path / "phi.bin", dtype=np.float64)
    uxa = vtp_array((tmp_path / "rs" / "b_p0_20.vtp").read_text(), "ux")
    restart = ("package gpu precision 64\n" + RESTART).replace("dump realgrid grid out 100 attributes 1 phi\n",
                                                            "dump fin atom/owned rs/c 10 attributes 2 x ux "
                                                            "decimalplaces 16 fmt e\n")
    (tmp_path / "in.phafd").write_text(restart)
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    assert "Saving on step 20" in r.stdout and "Saving on step 30" not in r.stdout
    phi_b = np.fromfile(tmp_path / "phi.bin", dtype=np.float64)
    uxb = vtp_array((tmp_path / "rs" / "c_p0_20.vtp").read_text(), "ux")
    assert np.linalg.norm(phi_b - phi_a) < 1e-10 * np.linalg.norm(phi_a)
    # unwrapped positions: the restart wraps every bead at its setup, the
    # uninterrupted run only at its neighbor rebuilds
    assert np.abs(uxb - uxa).max() < 1e-10 * np.abs(uxa).max()


@pytest.mark.parametrize("line", ["grid_populate flat_interface concentration 0.45 0.05 0.8 0.2 ${seed1}",
                                  "grid_populate sphere concentration 5.0 4.0 0.9 0.5"])
def test_populate_styles_parse(exe, tmp_path, line):
    scene(tmp_path, SCRIPT.replace("grid_populate constant concentration 0.5 0.02 ${seed1}", line))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr


def test_noise_state_commands(exe, tmp_path):
    """write_noise_state / read_noise_state: after the conjugate fix only."""
    scene(tmp_path, SCRIPT.replace("timestep 0", "read_noise_state ns.txt\ntimestep 0"))
    (tmp_path / "ns.txt").write_text("5489")
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr
    scene(tmp_path, SCRIPT.replace("fix atom/semiflexible", "write_noise_state ns.txt\nfix atom/semiflexible"))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and "noise state needs fix grid/conjugate/volfrac" in r.stderr
    scene(tmp_path, SCRIPT.replace("timestep 0", "read_noise_state none.txt\ntimestep 0"))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and "Cannot open file none.txt" in r.stderr


FTDUMP = SCRIPT.replace("dump realgrid grid out 100 attributes 1 phi\n",
                        "compute complex sk ft_phi norm\n"
                        "compute complex mu ft_chempot real\n"
                        "compute grid/cluster cl phi 0.5 gt\n"
                        "dump spec ftgrid ft/spec 10 attributes 2 c_sk c_mu\n"
                        "dump fields grid ft/fields 10 attributes 2 phi c_cl\n")


def test_compute_and_ftgrid_commands_parse(exe, tmp_path):
    scene(tmp_path, FTDUMP)
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 0, r.stderr
    assert r.stderr == ""


@pytest.mark.parametrize("edit,msg", [
    (("compute complex sk ft_phi norm", "compute sk complex ft_phi norm"), "Invalid compute."),
    (("compute complex sk ft_phi norm", "compute complex sk phi norm"), "Invalid array to compute in compute modulus."),
    (("compute complex sk ft_phi norm", "compute complex sk ft_phi square"), "Invalid argument in compute complex."),
    (("compute complex mu ft_chempot real", "compute complex sk ft_chempot real"), "Duplicate of compute sk."),
    (("attributes 2 c_sk c_mu", "attributes 2 c_sk c_cl"), "Cannot write dump, compute ID clis not a per_ftgrid quantity."),
    (("attributes 2 c_sk c_mu", "attributes 2 c_sk phi"), "Something wrong, should not get here."),
    (("attributes 2 phi c_cl", "attributes 2 phi c_sk"), "Cannot write dump, compute ID skis not a per_grid quantity."),
    (("attributes 2 c_sk c_mu", "attributes 2 c_sk c_none"), "Cannot write dump, compute ID nonedoesn't exist."),
])
def test_compute_and_ftgrid_errors(exe, tmp_path, edit, msg):
    """compute.cpp / compute_complex.cpp / dump.cpp:870-990 messages (dry run)."""
    scene(tmp_path, FTDUMP.replace(*edit))
    r = run(exe, tmp_path, "-sf", "gpu", "-dry-run")
    assert r.returncode == 1 and msg in r.stderr, r.stderr

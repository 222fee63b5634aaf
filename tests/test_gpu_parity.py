"""CUDA path against the FP64 oracle, through the C ABI (libphafd_gpu.so).

Tolerances: FP64 path 1e-10 relative (field and bead positions), FP32 path
2e-5 relative on single transforms; neighbor lists bit-exact as sets.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from phafd_gb300 import workloads as W
from tests.helpers import canon_grid, canon_half, rel_err, sk_rel_err, small_scene

pytestmark = pytest.mark.gpu


def gpu(precision=64, schedule="resident"):
    from phafd_gb300.gpu import PhafdGPU
    return PhafdGPU(precision=precision, schedule=schedule)


@pytest.mark.parametrize("precision,tol", [(64, 1e-12), (32, 2e-5)])
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 32, 32), (64, 64, 64), (16, 32, 64), (96, 32, 160), (128, 16, 16)])
def test_gradient_matches_oracle(gpu_lib, precision, tol, shape):
    nz, ny, nx = shape
    rng = np.random.default_rng(nx + 7 * ny + 13 * nz)
    phi = 0.4 + 0.1 * rng.standard_normal(shape)
    L = [nx * 0.7, ny * 1.1, nz * 0.9]
    o = Oracle(); g = gpu(precision)
    for d in (o, g):
        d.domain([-1.0, -2.0, -3.0], L)
        d.grid_style(nx, ny, nz)
        d.grid_set("phi", phi)
        d.stage_gradient()
    for f in ("gradx", "grady", "gradz"):
        assert rel_err(g.grid_get(f), o.grid_get(f)) < tol, f


@pytest.mark.parametrize("zghost", ["periodic", "rank1"])
def test_neighbor_lists_match_oracle_as_sets(gpu_lib, zghost):
    o = Oracle(); g = gpu(64)
    for d in (o, g):
        small_scene(d, n=32, L=32.0, nbeads=600, zghost=zghost, seed=11)
        d.setup()
    assert canon_half(g.half_list()) == canon_half(o.half_list())
    assert canon_grid(g.grid_list()) == canon_grid(o.grid_list())


@pytest.mark.parametrize("style", ["gaussian", "LJish", "LJish/linear"])
def test_pair_forces_and_deposit_match_oracle(gpu_lib, style):
    o = Oracle(); g = gpu(64)
    for d in (o, g):
        small_scene(d, n=32, L=32.0, nbeads=300, style=style, seed=5, amp=0.3)
        d.setup()
        d.stage_gradient()
        d.stage_borders_and_build()
        d.stage_pairs()
    _, _, fo, _ = o.atoms_get()
    _, _, fg, _ = g.atoms_get()
    assert rel_err(fg, fo) < 1e-12
    assert rel_err(g.grid_get("chempot"), o.grid_get("chempot")) < 1e-12


def _full_scene(d, noise, zghost="periodic", chi=2.5, steps_dt=5e-4):
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg["field_noise"] = noise
    cfg["dt"] = steps_dt
    cfg["bead_temp"] = 1.0 if noise != "off" else 0.0
    cfg["chi"] = chi
    W.apply(d, cfg, zghost=zghost)
    return cfg


@pytest.mark.parametrize("schedule", ["reference", "resident"])
@pytest.mark.parametrize("noise", ["off", "reference", "philox"])
def test_fp64_steps_match_oracle(gpu_lib, schedule, noise):
    o = Oracle(); g = gpu(64, schedule)
    for d in (o, g):
        _full_scene(d, noise)
        d.setup()
        d.run(30)
    xo, uxo, fo, imo = o.atoms_get()
    xg, uxg, fg, img = g.atoms_get()
    assert np.array_equal(imo, img)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 1e-10
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()
    assert np.abs(uxg - uxo).max() < 1e-10 * np.abs(uxo).max()
    assert rel_err(fg, fo) < 1e-9
    co, cg = o.counters(), g.counters()
    assert cg["neighbor_calls"] == co["neighbor_calls"]
    assert (cg["num_less_zero"], cg["num_great_zero"]) == (co["num_less_zero"], co["num_great_zero"])


@pytest.mark.parametrize("zghost", ["rank1", "periodic"])
def test_fp64_drag_fix_matches_oracle(gpu_lib, zghost):
    o = Oracle(); g = gpu(64, "reference")
    for d in (o, g):
        cfg = dict(W.CONFIGS["32cube_64beads"])
        W.apply(d, cfg, semiflexible=False, drag=1.0, zghost=zghost)
        d.setup()
        d.run(25)
    xo, *_ = o.atoms_get()
    xg, *_ = g.atoms_get()
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 1e-10


def test_fp32_path_error_against_oracle(gpu_lib):
    """FP32 production path vs the FP64 oracle: max |dphi| and the relative
    shell-averaged S(k) error, within the 1e-5 the FP32 path is held to."""
    o = Oracle(); g = gpu(32, "resident")
    for d in (o, g):
        _full_scene(d, "philox")
        d.setup()
        d.run(30)
    po, pg = o.grid_get("phi"), g.grid_get("phi")
    assert np.abs(pg - po).max() < 1e-5
    assert sk_rel_err(pg, po) < 1e-5


def test_fp32_mass_mode_exact(gpu_lib):
    g = gpu(32, "resident")
    _full_scene(g, "philox")
    g.setup()
    m0 = g.grid_get("ft_phi")[0, 0, 0]
    g.run(40)
    assert g.grid_get("ft_phi")[0, 0, 0] == m0


def test_nan_is_reported(gpu_lib):
    g = gpu(64, "resident")
    cfg = dict(W.CONFIGS["32cube_64beads"])
    W.apply(g, cfg)
    phi = np.full((32, 32, 32), 0.5)
    phi[3, 4, 5] = np.nan
    g.grid_set("phi", phi)
    g.setup()
    from phafd_gb300.gpu import PhafdError
    with pytest.raises(PhafdError, match="NAN"):
        g.run(2)


def test_neighbor_overflow_is_reported(gpu_lib):
    g = gpu(64)
    g.domain([0.0] * 3, [16.0] * 3)
    g.grid_style(16, 16, 16)
    g.grid_populate_constant(0.5, 0.0, 1)
    rng = np.random.default_rng(0)
    x = 8.0 + 0.4 * rng.random((200, 3))  # 200 beads inside one cutoff sphere
    n = len(x)
    g.atoms_create(np.arange(1, n + 1), np.zeros(n), np.zeros(n), x)
    g.pair_lj_cut(2 ** (1 / 6), 1.0, 1.0)
    g.neighbor(0.3)
    from phafd_gb300.gpu import PhafdError
    with pytest.raises(PhafdError, match="overflow"):
        g.setup()


def test_64cube_200beads_1000_steps_fp64(gpu_lib):
    """The FP64 parity workload: 64^3 grid, one 200-bead chain, noise off,
    1000 steps of dt = 1e-4: per-node phi and per-bead positions within 1e-10
    relative of the oracle, total concentration conserved."""
    cfg = W.CONFIGS["64cube_200beads"]
    o = Oracle(); g = gpu(64, "resident")
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
    m0 = o.grid_get("phi").sum()
    for d in (o, g):
        d.run(cfg["steps"])
    po, pg = o.grid_get("phi"), g.grid_get("phi")
    xo, uxo, _, _ = o.atoms_get()
    xg, uxg, _, _ = g.atoms_get()
    assert rel_err(pg, po) < 1e-10
    assert np.abs(uxg - uxo).max() < 1e-10 * np.abs(uxo).max()
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()
    assert abs(pg.sum() - m0) < 1e-10 * abs(m0)


@pytest.mark.parametrize("plane", [False, True])
@pytest.mark.parametrize("precision,n,tol", [(64, 128, 1e-10), (32, 128, 2e-5), (32, 256, 2e-5), (64, 256, 1e-10)])
def test_plane_fused_steps_match_oracle(gpu_lib, precision, n, tol, plane):
    """The resident step at sizes where the x and y passes run plane-fused
    (thread-block clusters exchanging a z-plane through distributed shared
    memory) against the oracle, three steps with device-generated noise."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(n=n, L=float(n), origin=-n / 2.0, nchains=4, chain_len=50, field_noise="philox", bead_temp=1.0,
               dt=1e-4)
    o = Oracle(); g = gpu(precision, "resident")
    g.set_plane_fusion(plane)
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(3)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < tol
    # the resident state holds grad phi of the current phi; the oracle's
    # arrays hold it from the start of the last step: recompute them
    o.stage_gradient()
    for f in ("gradx", "grady", "gradz"):
        assert rel_err(g.grid_get(f), o.grid_get(f)) < (tol if precision == 64 else 1e-4), f
    xo = o.atoms_get()[0]
    xg = g.atoms_get()[0]
    assert np.abs(xg - xo).max() < (1e-10 if precision == 64 else 1e-6) * np.abs(xo).max()


@pytest.mark.parametrize("zghost", ["periodic", "rank1"])
def test_fp32_lists_are_tight_supersets(gpu_lib, zghost):
    """FP32 contexts build their lists in FP32 with a 1e-5 relative cutoff
    margin: every exact pair is present and extras are at most a trace."""
    o = Oracle(); g = gpu(32)
    for d in (o, g):
        small_scene(d, n=32, L=32.0, nbeads=600, zghost=zghost, seed=11)
        d.setup()
    for got, want in ((canon_half(g.half_list()), canon_half(o.half_list())),
                      (canon_grid(g.grid_list()), canon_grid(o.grid_list()))):
        assert want <= got
        assert len(got - want) <= max(2, len(want) // 1000)


@pytest.mark.parametrize("shape", [(512, 16, 16), (16, 16, 512)])
def test_fp64_field_steps_with_512_point_axes(gpu_lib, shape):
    """512-point transforms (wider z tiles, x rows) against the oracle."""
    nz, ny, nx = shape
    o = Oracle(); g = gpu(64, "resident")
    for d in (o, g):
        d.domain([-nx / 2, -ny / 2, -nz / 2], [float(nx), float(ny), float(nz)])
        d.grid_style(nx, ny, nz)
        d.grid_populate_constant(0.45, 0.02, 3)
        d.fix_conjugate_volfrac(11, mobility=1.0, temp=0.01, volFH=1.0, gamma=100.0, noise="philox")
        d.fix_floryhuggins(temp=1.0, volFH=1.0, chi=3.0)
        d.set_dt(1e-4)
        d.setup()
        d.run(5)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 1e-10


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("style", ["flat_interface", "sphere"])
def test_populate_styles_match_oracle(gpu_lib, precision, style):
    """grid_populate flat_interface / sphere: host-generated phi uploaded to
    the context equals the oracle's (FP32 contexts hold its rounding)."""
    o = Oracle(); g = gpu(precision)
    for d in (o, g):
        d.domain([-8.0, -5.0, -6.0], [16.0, 10.0, 12.0])  # anisotropic spacing
        d.grid_style(32, 16, 16)
        if style == "flat_interface":
            d.grid_populate_flat_interface(0.45, 0.05, 0.8, 0.2, 7)
        else:
            d.grid_populate_sphere(3.5, 2.0 ** 0.5, 0.9, 0.3)
    want = o.grid_get("phi")
    got = g.grid_get("phi")
    # the library's host code may contract multiply-adds (the oracle is built
    # without): a few ulps in FP64; FP32 holds the rounding (half an ulp below 1)
    assert np.abs(got - want).max() < (1e-14 if precision == 64 else 6e-8)



@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 2e-5)])
def test_generic_256_point_plan_matches_oracle(gpu_lib, precision, tol):
    """The shared-memory tile transforms on 256-point axes (the autotuner's
    alternative to the register-resident ones) against the oracle."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(n=256, L=256.0, origin=-128.0, nchains=4, chain_len=50, field_noise="philox", bead_temp=1.0,
               dt=1e-4)
    o = Oracle(); g = gpu(precision, "resident")
    g.set_variants(generic256=True)
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(3)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < tol
    o.stage_gradient()
    for f in ("gradx", "grady", "gradz"):
        assert rel_err(g.grid_get(f), o.grid_get(f)) < (tol if precision == 64 else 1e-4), f


def _field_run(nx, ny, nz, tma, schedule="resident", steps=3):
    g = gpu(32, schedule)
    g.domain([-nx / 2, -ny / 2, -nz / 2], [float(nx), float(ny), float(nz)])
    g.grid_style(nx, ny, nz)
    g.grid_populate_constant(0.4, 0.02, 5)
    g.fix_gradphi(once=False)
    g.fix_conjugate_volfrac(15, mobility=1.0, temp=0.01, volFH=1.0, gamma=100.0, noise="philox")
    g.fix_floryhuggins(temp=1.0, volFH=1.0, chi=3.0)
    g.set_dt(1e-3)
    g.set_timestep(0)
    g.set_variants(xc2r_tma=tma, xr2c_tma=tma)
    g.setup()
    g.run(steps)
    out = {f: g.grid_get(f) for f in ("phi", "gradx", "grady", "gradz")}
    out["counters"] = np.array([g.counters()[k] for k in ("num_less_zero", "num_great_zero")])
    g.close()
    return out


@pytest.mark.parametrize("shape,schedule", [((256, 256, 256), "resident"), ((256, 64, 32), "resident"),
                                            ((256, 64, 32), "reference")])
def test_tma_fed_x_passes_equal_register_resident(gpu_lib, shape, schedule):
    """The tensor-map fed persistent x r2c and x c2r (PHAFD_TUNE_XR2C_TMA,
    PHAFD_TUNE_XC2R_TMA) form the same lines and run the same transforms as
    the register-resident x passes that load their own tiles: without beads
    (no floating-point atomics anywhere in the step) phi, the three
    gradients and the Flory-Huggins reflection counters after three steps
    are bit-identical.  The reference schedule adds the plain r2c of phi
    (no Flory-Huggins prologue) to every step."""
    a = _field_run(*shape, tma=False, schedule=schedule)
    b = _field_run(*shape, tma=True, schedule=schedule)
    for f in a:
        if f != "counters":
            assert np.abs(a[f]).max() > 0, f
        assert np.array_equal(a[f], b[f]), f


def test_tma_fed_x_passes_with_beads_match_oracle(gpu_lib):
    """The tensor-map fed x passes in a 256^3 FP32 step with chains (masked
    gradient stores, neighbor rebuilds) against the FP64 oracle."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(n=256, L=256.0, origin=-128.0, nchains=4, chain_len=50, field_noise="philox", bead_temp=1.0,
               dt=1e-4)
    o = Oracle(); g = gpu(32, "resident")
    g.set_variants(xc2r_tma=True, xr2c_tma=True)
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(3)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 2e-5
    xo, xg = o.atoms_get()[0], g.atoms_get()[0]
    assert np.abs(xg - xo).max() < 1e-5 * np.abs(xo).max()
    assert g.counters()["timestep"] == 3


def test_tma_x_r2c_reads_the_whole_deposit(gpu_lib):
    """The tensor-map fed x r2c reads the bead deposit only in the sectors of
    its support mask (rebuilt with the grid lists): the chempot it
    materialises (deposit + Flory-Huggins part) equals the one of the x r2c
    that reads the deposit everywhere, over steps that include neighbor
    rebuilds (the deposits' floating-point atomics differ in order only)."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(n=256, L=256.0, origin=-128.0, nchains=16, chain_len=200, field_noise="philox", bead_temp=1.0,
               dt=1e-3)
    out = []
    chains = None
    for tma in (False, True):
        g = gpu(32, "resident")
        chains = W.apply(g, cfg, chains=chains)
        g.set_keep_chempot(True)
        g.set_variants(xc2r_tma=True, xr2c_tma=tma)
        g.setup()
        g.run(6)
        out.append((g.grid_get("chempot"), g.counters()["neighbor_calls"]))
        g.close()
    (a, na), (b, nb) = out
    assert na == nb and na >= 2
    assert np.abs(b - a).max() < 1e-5 * np.abs(a).max()


@pytest.mark.parametrize("graph_steps", [2, 8, 16])
def test_graph_length_does_not_change_the_run(gpu_lib, graph_steps):
    """Runs of 19 steps (8- or 16-step graphs, whose later steps check their
    neighbor lists on the previous step's bead branch, then 2- and 1-step
    graphs) match the oracle within 1e-10, lists included."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(field_noise="philox", bead_temp=1.0, dt=1e-3)
    o = Oracle(); g = gpu(64, "resident")
    g.set_graph_steps(graph_steps)
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(19)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 1e-10
    xo, xg = o.atoms_get()[0], g.atoms_get()[0]
    assert np.abs(xg - xo).max() < 1e-10 * np.abs(xo).max()
    assert g.counters()["neighbor_calls"] == o.counters()["neighbor_calls"] >= 2
    assert canon_half(g.half_list()) == canon_half(o.half_list())
    assert canon_grid(g.grid_list()) == canon_grid(o.grid_list())
    with pytest.raises(Exception):
        g.set_graph_steps(3)


def test_pipelined_bead_readback(gpu_lib):
    """phafd_atoms_get_async / phafd_wait_slot: every step's beads read back
    while the next step is already enqueued equal a step-by-step run with
    blocking reads (page-locked buffers, two slots alternating)."""
    from phafd_gb300 import gpu as G
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(field_noise="philox", bead_temp=1.0, dt=1e-3)
    a = gpu(64, "resident"); b = gpu(64, "resident")
    chains = None
    for d in (a, b):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
    n = a.n
    bufs = [(np.empty((n, 3)), np.empty((n, 3)), np.empty((n, 3)), np.empty(n, np.int32)) for _ in range(2)]
    for bb in bufs:
        for arr in bb:
            G.host_register(arr)
    got = []
    steps = 7
    for s in range(steps):
        a.run_async(1)
        a.atoms_get_async(bufs[s & 1], s & 1)
        if s:
            a.wait_slot((s - 1) & 1)
            got.append([arr.copy() for arr in bufs[(s - 1) & 1]])
    a.wait_slot((steps - 1) & 1)
    got.append([arr.copy() for arr in bufs[(steps - 1) & 1]])
    for bb in bufs:
        for arr in bb:
            G.host_unregister(arr)
    for s in range(steps):
        b.run(1)
        want = b.atoms_get()
        for g_, w_ in zip(got[s], want):
            assert np.allclose(g_, w_, rtol=1e-12, atol=1e-12), s
    assert not np.array_equal(got[0][0], got[-1][0])  # the beads moved
    with pytest.raises(Exception):
        a.wait_slot(3)  # nothing enqueued there


def test_autotune_steps_are_steps_of_the_run(gpu_lib):
    """The autotuner times each variant on the run's own steps: afterwards
    the state equals the oracle's after the same number of steps, and the
    fastest variant is kept."""
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(n=64, L=64.0, origin=-32.0, nchains=2, chain_len=40, field_noise="philox", bead_temp=1.0,
               dt=1e-4)
    o = Oracle(); g = gpu(64, "resident")
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
    best, ms = g.autotune(steps=2)
    assert ms[0] > 0 and ms[1] > 0      # separate and plane-fused passes (64 x 64 planes)
    assert ms[2] < 0 and ms[3] < 0      # no 256-point axis
    assert (ms[4:] < 0).all()           # the tensor-map x c2r: FP32 with Nx = 256 only
    assert best == int(np.argmin(np.where(ms > 0, ms, np.inf)))
    done = g.counters()["timestep"]
    assert done == 2 * (4 + 2)
    o.run(done)
    g.run(3)
    o.run(3)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < 1e-10
    assert np.abs(g.atoms_get()[0] - o.atoms_get()[0]).max() < 1e-10 * np.abs(o.atoms_get()[0]).max()


@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 2e-5)])
def test_512cube_steps_match_oracle(gpu_lib, precision, tol):
    """The largest single-GPU grid (512^3, box 512) against the oracle: three
    steps with Philox field and bead noise and four 50-bead chains (the
    oracle's all-node grid list at this size allows few beads in a test)."""
    from oracle import oracle as OR
    cfg = dict(W.CONFIGS["512cube_1Mbeads"])
    cfg.update(nchains=4, chain_len=50)
    OR.set_threads(OR.host_threads())
    o = Oracle(); g = gpu(precision, "resident")
    chains = None
    for d in (o, g):
        chains = W.apply(d, cfg, chains=chains)
        d.setup()
        d.run(3)
    assert rel_err(g.grid_get("phi"), o.grid_get("phi")) < tol
    xo = o.atoms_get()[0]
    xg = g.atoms_get()[0]
    assert np.abs(xg - xo).max() < (1e-10 if precision == 64 else 1e-6) * np.abs(xo).max()
    assert g.counters()["neighbor_calls"] == o.counters()["neighbor_calls"]

"""Resume with the reference noise's generator state, and the spectra the
compute complex command reads, against the oracle (FP64, resident schedule).

compute complex ft_phi is the unnormalised spectrum of the current phi times
1/(dx dy dz) (compute_complex.cpp:50-91): checked against the oracle's r2c of
its own phi.  ft_chempot and the real chempot are the last step's mu, kept
only when phafd_set_keep_chempot precedes the steps; without it a read after
a run is refused.  Placed after the other GPU files so that a failure here
leaves their results in place."""
import numpy as np
import pytest

from oracle import oracle as OR
from oracle.oracle import Oracle
from phafd_gb300 import workloads as W
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def gpu(precision=64):
    from phafd_gb300.gpu import PhafdGPU
    return PhafdGPU(precision=precision, schedule="resident")


def test_reference_noise_resume_matches_uninterrupted_run(gpu_lib):
    """FP64, reference noise: a context restored from phi, wrapped positions,
    image flags, timestep and the host generator's state continues the run."""
    cfg = dict(W.CONFIGS["32cube_64beads"], field_noise="reference", dt=5e-4)
    a = gpu(64)
    chains = W.apply(a, cfg)
    a.setup()
    a.run(10)
    phi10, state = a.grid_get("phi"), a.noise_state()
    x10, _, _, im10 = a.atoms_get()
    a.run(10)
    b = gpu(64)
    W.apply(b, cfg, chains=(x10.copy(),) + tuple(chains[1:]), phi=phi10)
    b.atoms_set_images(im10.copy())
    b.set_noise_state(state)
    b.set_timestep(10)
    b.setup()
    b.run(10)
    pa = a.grid_get("phi")
    assert rel_err(b.grid_get("phi"), pa) < 1e-10
    assert np.abs(b.atoms_get()[1] - a.atoms_get()[1]).max() < 1e-10 * np.abs(a.atoms_get()[1]).max()


def _scene(d, keep):
    cfg = dict(W.CONFIGS["32cube_64beads"], field_noise="philox", bead_temp=1.0, dt=5e-4)
    if keep:
        d.set_keep_chempot(True)
    W.apply(d, cfg)
    d.setup()
    d.run(6)
    return cfg


def test_chempot_after_a_run_needs_keep_chempot(gpu_lib):
    from phafd_gb300.gpu import PhafdError
    g = gpu()
    _scene(g, keep=False)
    for field in ("chempot", "ft_chempot"):
        with pytest.raises(PhafdError, match="keep_chempot"):
            g.grid_get(field)
    g.grid_get("phi")  # the rest stays readable


def test_chempot_and_spectra_match_oracle(gpu_lib):
    o, g = Oracle(), gpu()
    cfg = _scene(g, keep=True)
    _scene(o, keep=False)  # the oracle always keeps mu
    assert rel_err(g.grid_get("chempot"), o.grid_get("chempot")) < 1e-9
    assert rel_err(g.grid_get("ft_chempot"), o.grid_get("ft_chempot")) < 1e-9
    n = cfg["n"]
    prefac = 1.0 / (cfg["L"] / n) ** 3
    spec = OR.fft_r2c(o.grid_get("phi"))  # [ky][kz][kx], unnormalised
    want = {"real": spec.real * prefac, "imag": spec.imag * prefac, "modulus": np.abs(spec) * prefac,
            "norm": np.abs(spec) ** 2 * prefac ** 2}
    for q, w in want.items():
        assert rel_err(g.compute_complex("ft_phi", q), w) < 1e-9, q
    mu_spec = o.grid_get("ft_chempot")
    assert rel_err(g.compute_complex("ft_chempot", "norm"), np.abs(mu_spec) ** 2 * prefac ** 2) < 1e-9


from tests.test_host_script import FTDUMP, exe, run, scene  # noqa: E402,F401  (exe is a fixture)


def _appended(path, narrays):
    raw = path.read_bytes()
    head = raw[:raw.index(b'<AppendedData encoding="raw">')].decode()
    at = raw.index(b'<AppendedData encoding="raw">\n_') + len(b'<AppendedData encoding="raw">\n_')
    out = []
    for _ in range(narrays):
        nbytes = int.from_bytes(raw[at:at + 4], "little")
        out.append(np.frombuffer(raw, "<f8", nbytes // 8, at + 4))
        at += 4 + nbytes
    return head, out


def test_script_ftgrid_dump(exe, tmp_path, gpu_lib):
    """compute complex + ftgrid dump through a script: zeros in the starting
    dump (the reference's computes have not run yet), then the spectrum of
    the dump step's starting phi; its k = 0 mode carries the conserved mass
    of the initial field.  The grid dump's cluster labels match an
    independent labelling of the same step's phi."""
    from tests.cluster_ref import periodic_min_id_labels
    scene(tmp_path, FTDUMP)
    (tmp_path / "ft").mkdir()
    r = run(exe, tmp_path, "-sf", "gpu")
    assert r.returncode == 0, r.stderr
    head, (sk0, mu0) = _appended(tmp_path / "ft" / "spec_p0_0.vti", 2)
    assert 'WholeExtent="0 16 0 31 0  31"' in head and 'Origin="0 0 0 "' in head
    assert 'Spacing="0.19635 0.19635 0.19635 "' in head  # 2 * 3.141592 / 32
    assert not sk0.any() and not mu0.any()
    _, (phi0, cl0) = _appended(tmp_path / "ft" / "fields_p0_0.vti", 2)
    assert not cl0.any()
    _, (sk, mu) = _appended(tmp_path / "ft" / "spec_p0_10.vti", 2)
    assert sk.size == 17 * 32 * 32 and np.isfinite(sk).all() and (sk >= 0).all() and np.isfinite(mu).all()
    mass = phi0.sum()  # dx = dy = dz = 1: prefac 1
    assert abs(sk[0] - mass ** 2) < 1e-5 * mass ** 2
    assert np.abs(mu).max() > 0
    _, (phi10, cl10) = _appended(tmp_path / "ft" / "fields_p0_10.vti", 2)
    want, _ = periodic_min_id_labels(phi10.reshape(32, 32, 32), 0.5, True)
    assert np.array_equal(cl10.astype(np.int64), want.ravel().astype(np.int64))


def test_step_start_spectrum_is_the_previous_phi(gpu_lib):
    """PHAFD_FIELD_FT_PHI_STEP_START after 6 steps: the r2c of phi after 5
    (the oracle's), zeros right after set-up."""
    cfg = dict(W.CONFIGS["32cube_64beads"], field_noise="philox", bead_temp=1.0, dt=5e-4)
    o, g = Oracle(), gpu()
    chains = W.apply(g, cfg)
    W.apply(o, cfg, chains=chains)
    g.setup()
    o.setup()
    assert not g.grid_get("ft_phi_step_start").any()
    o.run(5)
    want = OR.fft_r2c(o.grid_get("phi"))
    g.run(6)
    assert rel_err(g.grid_get("ft_phi_step_start"), want) < 1e-9
    g.run(1)  # a single step (the other graph path)
    o.run(1)
    assert rel_err(g.grid_get("ft_phi_step_start"), OR.fft_r2c(o.grid_get("phi"))) < 1e-9


def test_fp64_run_matches_golden_fixture(gpu_lib):
    """The CUDA FP64 path on the committed oracle fixture's inputs (16^3
    grid, 12-bead chain, Philox noise, 10 steps): the parity tolerance."""
    import os
    from tests.golden.make_golden import step_case
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_cases.npz"))
    phi, x, ux, f, im = step_case(gpu(64), g["phi0"], (g["x0"], g["tags"], g["mol"], g["types"]))
    assert rel_err(phi, g["phi"]) < 1e-10
    assert np.abs(ux - g["ux"]).max() < 1e-10 * np.abs(g["ux"]).max()
    assert np.array_equal(im, g["images"])

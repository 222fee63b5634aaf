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

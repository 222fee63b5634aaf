"""Macro-step machinery of the learned propagator on the GPU: the
K-substep linearised update, the bead density, S(k), state copies, mass
conservation and what the trained network gains over the linearised step."""
import numpy as np
import pytest

from phafd_gb300 import surrogate as S
from phafd_gb300 import workloads as W
from phafd_gb300.gpu import PhafdGPU

pytestmark = pytest.mark.gpu


def small_cfg(noise="off"):
    c = dict(W.CONFIGS["32cube_64beads"])
    c["field_noise"] = noise
    return c


def field_only(n=32, fh=False, noise="off"):
    g = PhafdGPU(precision=32, schedule="resident")
    g.domain([-n / 2] * 3, [float(n)] * 3)
    g.grid_style(n, n, n)
    g.grid_populate_constant(0.45, 0.02, 3)
    g.fix_conjugate_volfrac(11, mobility=1.0, temp=0.01, volFH=1.0, gamma=100.0, noise=noise)
    if fh:
        g.fix_floryhuggins(temp=1.0, volFH=1.0, chi=3.0)
    g.set_dt(1e-4)
    return g


def test_one_substep_is_the_plain_step(gpu_lib):
    a, b = field_only(fh=True), field_only(fh=True)
    b.set_linear_substeps(1, 123.0)
    a.run(7)
    b.run(7)
    assert np.array_equal(a.grid_get("phi"), b.grid_get("phi"))


def test_macro_step_equals_k_steps_of_a_linear_model(gpu_lib):
    # without Flory-Huggins and beads the plain update is linear in phi
    a, b = field_only(), field_only()
    b.set_linear_substeps(20, 0.0)
    a.run(20)
    b.run(1)
    pa, pb = a.grid_get("phi"), b.grid_get("phi")
    d = pa - pa.mean()
    assert np.linalg.norm(pb - pa) / np.linalg.norm(d) < 1e-4


def test_density_matches_brute_force(gpu_lib):
    import torch
    cfg = small_cfg()
    g = PhafdGPU(precision=32, schedule="resident")
    W.apply(g, cfg)
    g.setup()
    rho = torch.empty(g.shape, device="cuda")
    g.deposit_density(rho.data_ptr())
    got = rho.cpu().numpy().astype(np.float64)
    x, *_ = g.atoms_get()
    n, L, lo = cfg["n"], cfg["L"], cfg["origin"]
    want = np.zeros((n, n, n))
    ax = lo + np.arange(n) * (L / n)
    for p in x:
        d = [((ax - p[k] + L / 2) % L) - L / 2 for k in range(3)]
        r2 = d[2][:, None, None] ** 2 + d[1][None, :, None] ** 2 + d[0][None, None, :] ** 2
        s = r2 / cfg["ga_cut"] ** 2
        want += np.where(s <= 1.0, (np.exp(-s / 2) - np.exp(-0.5)) * np.exp(0.5), 0.0)
    assert np.abs(got - want).max() < 1e-4 * max(1.0, want.max())


def test_structure_factor_matches_numpy(gpu_lib):
    g = field_only(n=32)
    g.run(3)
    nb = 16
    sk, cnt = g.structure_factor(nb)
    phi = g.grid_get("phi")
    F = np.fft.fftn(phi)
    q = [np.fft.fftfreq(32) * 32 for _ in range(3)]
    kz, ky, kx = np.meshgrid(*q, indexing="ij")
    b = np.floor(np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)).astype(int)
    want = np.zeros(nb)
    wc = np.zeros(nb, np.int64)
    p = np.abs(F) ** 2
    for k in range(nb):
        m = (b == k)
        m[0, 0, 0] = False
        wc[k] = m.sum()
        want[k] = p[m].sum() / max(m.sum(), 1) / phi.size
    assert np.array_equal(cnt, wc)
    assert np.allclose(sk, want, rtol=2e-4, atol=0)


def test_copy_state_continues_identically(gpu_lib):
    cfg = small_cfg("philox")
    a = PhafdGPU(precision=32, schedule="resident")
    ch = W.apply(a, cfg)
    a.setup()
    a.run(5)
    b = PhafdGPU(precision=32, schedule="resident")
    W.apply(b, cfg, chains=ch)
    b.setup()
    b.copy_state_from(a)
    a.run(6)
    b.run(6)
    # FP32 deposit atomics make the two runs differ at round-off level only
    pa, pb = a.grid_get("phi"), b.grid_get("phi")
    assert np.abs(pa - pb).max() < 1e-6
    assert np.abs(a.atoms_get()[0] - b.atoms_get()[0]).max() < 1e-6


def test_macro_step_with_network_conserves_mass(gpu_lib):
    import torch
    cfg = S.traj_cfg(128, 2000, 3.0, 0.42, 5)
    ch = S.make_chains([cfg], 1)[0]
    s = S.sim(cfg, ch, noise=True)
    from phafd_gb300.fno import init_params
    net = S.new_network(s.shape, params=init_params(1, out_scale=1.0))
    net.set_norm(np.array([0.42, 0.02, 0.0, 1.0, 3.0, 0.3, 1e-3, 0.0], np.float32))
    m0 = S.mean_phi(s)
    s.set_linear_substeps(20, S.fh_f2(3.0, 0.42))
    rho = torch.empty(s.shape, device="cuda")
    corr = torch.empty(s.shape, device="cuda")
    for _ in range(3):
        s.deposit_density(rho.data_ptr())
        net.infer(s.grid_device("phi"), rho.data_ptr(), 3.0, corr.data_ptr())
        assert float(corr.abs().max()) > 0
        s.run(1)
        s.grid_add_device(corr.data_ptr(), 1.0)
    assert abs(S.mean_phi(s) - m0) < 2e-6
    s.close()
    net.close()


def test_trained_network_beats_the_linearised_step(gpu_lib):
    """A short training on a few 128^3 trajectories reduces the macro-step
    error below the linearised step's on held-out states."""
    rng = np.random.default_rng(0)
    specs = [(128, int(rng.integers(4000, 16001)), rng.uniform(2.5, 3.5), rng.uniform(0.35, 0.5), 100 + i)
             for i in range(6)]
    data = S.generate(specs[:4], samples=2, burn=60, gap=40, workers=4)
    held = S.generate(specs[4:], samples=1, burn=60, workers=2)
    net = S.new_network((128, 128, 128), train=True, seed=3)
    net.set_norm(S.norm_from(*data))
    assert S.gain(net, data) == pytest.approx(1.0)  # the correction starts at zero
    S.train(net, data, epochs=20, lr=1e-3, batch=2)
    g_train, g_held = S.gain(net, data), S.gain(net, held)
    assert g_train < 0.99 and g_held < 1.0, (g_train, g_held)
    net.close()

"""Learned propagator on the GPU against its CPU oracle: tensor-core operand
layouts, forward, gradients, a training run, mass conservation."""
import numpy as np
import pytest

from oracle.fno_oracle import FNOOracle, bf16
from phafd_gb300 import fno as F

pytestmark = pytest.mark.gpu

NORM = np.array([0.45, 0.05, 0.0, 1.0, 3.0, 0.3, 1.0, 0.0], np.float32)


def dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a, np.float32), device="cuda")


def scene(shape, seed=1):
    rng = np.random.default_rng(seed)
    phi = (0.45 + 0.05 * rng.standard_normal(shape)).astype(np.float32)
    rho = (np.abs(rng.standard_normal(shape)) * (rng.random(shape) < 0.05)).astype(np.float32)
    tgt = (0.3 * rng.standard_normal(shape)).astype(np.float32)
    return phi, rho, tgt


def params(seed):
    p = F.init_params(seed, out_scale=1.0)
    # spectral weights large enough that the Fourier branch matters
    for l in range(4):
        o, shp = F.layout()["R%d" % l]
        n = int(np.prod(shp))
        p[o:o + n] *= 64.0
    return p


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def test_tensor_core_layouts(gpu_lib):
    kmaj, mnmaj = F.selftest(0)
    assert kmaj and mnmaj


@pytest.mark.parametrize("shape", [(16, 16, 128), (16, 16, 256)])
def test_forward_matches_oracle(gpu_lib, shape):
    import torch
    phi, rho, _ = scene(shape)
    p = params(3)
    net = F.FNO(shape, train=False)
    net.set_params(p)
    net.set_norm(NORM)
    dphi, drho = dev(phi), dev(rho)
    corr = torch.zeros(shape, device="cuda")
    net.infer(dphi.data_ptr(), drho.data_ptr(), 3.1, corr.data_ptr())
    torch.cuda.synchronize()
    got = corr.cpu().numpy()
    want = FNOOracle(p, shape, NORM, bf=True).correction(phi, rho, 3.1)
    assert np.isfinite(got).all()
    assert rel(got, want) < 1e-2
    assert abs(got.astype(np.float64).mean()) < 1e-5 * np.abs(got).max()
    net.close()


def test_gradients_match_oracle(gpu_lib):
    shape = (16, 16, 128)
    phi, rho, tgt = scene(shape, 5)
    p = params(4)
    net = F.FNO(shape, train=True)
    net.set_params(p)
    net.set_norm(NORM)
    net.zero_grad()
    dphi, drho, dtgt = dev(phi), dev(rho), dev(tgt)  # kept alive while the library reads them
    loss = net.forward_backward(dphi.data_ptr(), drho.data_ptr(), 3.1, dtgt.data_ptr())
    g = net.get_grad()
    lo, go = FNOOracle(p, shape, NORM, bf=True).loss_and_grad(phi, rho, 3.1, tgt)
    gflat = FNOOracle.flat(go)
    errs = {}
    for name, (o, shp) in F.layout().items():
        n = int(np.prod(shp))
        errs[name] = rel(g[o:o + n], gflat[o:o + n])
    assert abs(loss - lo) < 1e-3 * lo and max(errs.values()) < 3e-2, (loss, lo, errs)
    net.close()


def test_training_reduces_loss(gpu_lib):
    """Fit a target that is a smooth functional of phi and rho."""
    import torch
    shape = (16, 16, 128)
    rng = np.random.default_rng(9)
    net = F.FNO(shape, train=True)
    net.set_params(F.init_params(2, out_scale=0.1))
    net.set_norm(NORM)
    data = []
    for k in range(4):
        phi, rho, _ = scene(shape, 20 + k)
        # target: a local nonlinear response plus a smoothed copy of phi
        sm = np.real(np.fft.ifftn(np.fft.fftn(phi - phi.mean()) * np.exp(-0.5 * (np.add.outer(
            np.add.outer(np.fft.fftfreq(shape[0]) ** 2, np.fft.fftfreq(shape[1]) ** 2),
            np.fft.fftfreq(shape[2]) ** 2)) * 400)))
        t = 5 * (phi - 0.45) ** 2 + 10 * sm + 0.2 * rho
        data.append(tuple(dev(a) for a in (phi, rho, (t - t.mean()).astype(np.float32))))
    first = last = None
    for it in range(60):
        net.zero_grad()
        tot = 0.0
        for d in data:
            tot += net.forward_backward(d[0].data_ptr(), d[1].data_ptr(), 3.0, d[2].data_ptr())
        net.adam_step(2e-3, nbatch=len(data))
        if first is None:
            first = tot
        last = tot
    torch.cuda.synchronize()
    assert last < 0.5 * first, (first, last)
    net.close()

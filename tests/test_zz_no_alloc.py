"""phafd_gradphi_noalloc: the gradient for callers that cannot allocate.

A host code that owns the device heap (or forbids cudaMalloc/cudaFree in a
time step, where they would synchronise the device) passes phi and the three
outputs as its own device arrays; the library must allocate nothing and use
its built-in scratch array.  This file runs last so that a failure here comes
after every other test has run.  It checks the entry point against the
context-based gradient (phafd_stage_gradient) on two calls in a row, at the
FP64 transform tolerance of the other tests (1e-12 relative), and that a grid
beyond the built-in scratch size is refused.
"""
import numpy as np
import pytest

from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

PHAFD_ERR_UNSUPPORTED = -6


def context_gradient(phi, period):
    from phafd_gb300.gpu import PhafdGPU
    nz, ny, nx = phi.shape
    g = PhafdGPU(precision=64)
    g.domain([0.0, 0.0, 0.0], period)
    g.grid_style(nx, ny, nz)
    g.grid_set("phi", phi)
    g.stage_gradient()
    out = [g.grid_get(f) for f in ("gradx", "grady", "gradz")]
    g.close()
    return out


def test_noalloc_gradient_matches_context_gradient_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    from phafd_gb300.gpu import load
    L = load()
    rng = np.random.default_rng(2024)
    cases = [((32, 64, 16), [16 * 0.9, 64 * 1.1, 32 * 0.7]), ((16, 16, 64), [64.0, 16.0, 16.0])]
    for shape, period in cases:  # two calls in a row, the second on a different grid
        nz, ny, nx = shape
        phi = 0.4 + 0.1 * rng.standard_normal(shape)
        ref = context_gradient(phi, period)
        dev = torch.device("cuda", 0)
        t_phi = torch.tensor(phi, dtype=torch.float64, device=dev)
        outs = [torch.full(shape, float("nan"), dtype=torch.float64, device=dev) for _ in range(3)]
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = L.phafd_gradphi_noalloc(t_phi.data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(),
                                     nx, ny, nz, np.asarray(period, np.float64), stream)
        torch.cuda.synchronize(dev)
        assert rc == 0
        for got, want in zip(outs, ref):
            assert rel_err(got.cpu().numpy(), want) < 1e-12


def test_noalloc_refuses_grids_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    from phafd_gb300.gpu import load
    L = load()
    dev = torch.device("cuda", 0)
    shape = (16, 16, 128)
    t = torch.zeros(shape, dtype=torch.float64, device=dev)
    outs = [torch.full(shape, 7.0, dtype=torch.float64, device=dev) for _ in range(3)]
    rc = L.phafd_gradphi_noalloc(t.data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(),
                                 128, 16, 16, np.asarray([128.0, 16.0, 16.0]), None)
    torch.cuda.synchronize(dev)
    assert rc == PHAFD_ERR_UNSUPPORTED
    assert all(bool((o == 7.0).all()) for o in outs)  # nothing written

"""compute grid/cluster on the GPU against the oracle (exact integer labels)
and, at 128^3, against an independent connected-component labelling."""
import numpy as np
import pytest

from phafd_gb300.gpu import PhafdGPU
from tests.cluster_ref import periodic_min_id_labels, smooth_field
from tests.test_clusters_oracle import oracle_labels

pytestmark = pytest.mark.gpu


def gpu_labels(phi, threshold, cond, precision):
    nz, ny, nx = phi.shape
    g = PhafdGPU(precision=precision)
    g.domain([0.0, 0.0, 0.0], [float(nx), float(ny), float(nz)])
    g.grid_style(nx, ny, nz)
    g.grid_set("phi", phi)
    return g.compute_grid_clusters(threshold, cond)


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("shape", [(32, 32, 32), (16, 32, 64)])
@pytest.mark.parametrize("threshold,cond", [(0.55, "gt"), (0.45, "lt"), (0.5, "gt")])
def test_clusters_match_oracle(gpu_lib, precision, shape, threshold, cond):
    phi = smooth_field(shape, seed=7 + sum(shape))
    if precision == 32:
        phi = phi.astype(np.float32).astype(np.float64)  # the field the FP32 context holds
    got, n = gpu_labels(phi, threshold, cond, precision)
    want = oracle_labels(phi, threshold, cond)
    assert np.array_equal(got, want)
    assert n == len(np.unique(want[want >= 0]))


def test_clusters_at_128cube_match_independent_labelling(gpu_lib):
    phi = smooth_field((128, 128, 128), seed=3, width=4.0)
    got, n = gpu_labels(phi, 0.52, "gt", 64)
    want, nw = periodic_min_id_labels(phi, 0.52, True)
    assert np.array_equal(got, want)
    assert n == nw


def test_empty_and_full_sets(gpu_lib):
    phi = np.full((16, 16, 16), 0.5)
    got, n = gpu_labels(phi, 0.9, "gt", 64)
    assert n == 0 and (got == -1).all()
    got, n = gpu_labels(phi, 0.1, "gt", 64)
    assert n == 1 and (got == 0).all()

"""The oracle's compute grid/cluster (a restatement of the reference's label
sweeps) against an independent connected-component labelling."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tests.cluster_ref import periodic_min_id_labels, smooth_field


def oracle_labels(phi, threshold, cond):
    nz, ny, nx = phi.shape
    o = Oracle()
    o.domain([0.0, 0.0, 0.0], [float(nx), float(ny), float(nz)])
    o.grid_style(nx, ny, nz)
    o.grid_set("phi", phi)
    return o.compute_grid_clusters(threshold, cond)


@pytest.mark.parametrize("shape", [(16, 16, 16), (12, 16, 20)])
@pytest.mark.parametrize("threshold,cond", [(0.55, "gt"), (0.45, "lt"), (0.5, "gt")])
def test_oracle_clusters_match_periodic_components(shape, threshold, cond):
    phi = smooth_field(shape, seed=sum(shape))
    want, _ = periodic_min_id_labels(phi, threshold, cond == "gt")
    assert np.array_equal(oracle_labels(phi, threshold, cond), want)


def test_cluster_wrapping_every_face_is_one_cluster():
    phi = np.full((8, 8, 8), 0.3)
    phi[:, 3, 3] = 0.9   # a line through both z faces ...
    phi[3, :, 3] = 0.9   # ... crossing one through both y faces: one cluster
    phi[5, 5, :] = 0.9   # a separate line through both x faces
    got = oracle_labels(phi, 0.5, "gt")
    want, n = periodic_min_id_labels(phi, 0.5, True)
    assert np.array_equal(got, want)
    assert len(np.unique(got[got >= 0])) == n


def test_condition_must_be_lt_or_gt():
    o = Oracle()
    o.domain([0.0] * 3, [8.0] * 3)
    o.grid_style(8, 8, 8)
    with pytest.raises(ValueError):
        o.compute_grid_clusters(0.5, "ge")

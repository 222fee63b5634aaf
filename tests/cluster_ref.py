"""Independent labelling for the compute grid/cluster tests: scipy.ndimage
connected components (6-connectivity), merged across the periodic faces,
each component labelled with its smallest z + (y Nx + x) Ny."""
import numpy as np


def periodic_min_id_labels(phi, threshold, greater):
    from scipy import ndimage
    nz, ny, nx = phi.shape
    mask = phi > threshold if greater else phi < threshold
    lab, n = ndimage.label(mask)
    parent = np.arange(n + 1)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for axis in range(3):
        a = np.take(lab, 0, axis=axis)
        b = np.take(lab, -1, axis=axis)
        both = (a > 0) & (b > 0)
        for u, v in zip(a[both].tolist(), b[both].tolist()):
            ru, rv = find(u), find(v)
            if ru != rv:
                parent[max(ru, rv)] = min(ru, rv)
    roots = np.array([find(i) for i in range(n + 1)])
    comp = roots[lab]
    z, y, x = np.indices(phi.shape)
    ids = z + (y * nx + x) * ny
    big = np.iinfo(np.int64).max
    minid = np.full(n + 1, big, np.int64)
    np.minimum.at(minid, comp[mask], ids[mask])
    out = np.full(phi.shape, -1, np.int64)
    out[mask] = minid[comp[mask]]
    return out.astype(np.int32), len(np.unique(comp[mask]))


def smooth_field(shape, seed, width=3.0):
    """A periodic random field with structure several nodes wide."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kz, ky, kx = np.meshgrid(*k, indexing="ij")
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-0.5 * (kx ** 2 + ky ** 2 + kz ** 2) * (2 * np.pi * width) ** 2)))
    return 0.5 + 0.1 * f / f.std()

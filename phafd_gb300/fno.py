"""Host binding of the learned field propagator (include/phafd_fno.h).

The network runs only on the GPU through libphafd_gpu.so; there is no CPU
path.  Device buffers are passed as raw addresses (torch tensors' data_ptr()
or the context's own fields from PhafdGPU.grid_device)."""
import ctypes as C

import numpy as np

from .gpu import ERRORS, load

EXPORTS = [
    "phafd_fno_param_count", "phafd_fno_create", "phafd_fno_destroy", "phafd_fno_last_error",
    "phafd_fno_set_params", "phafd_fno_get_params", "phafd_fno_set_norm", "phafd_fno_infer",
    "phafd_fno_zero_grad", "phafd_fno_forward_backward", "phafd_fno_get_grad", "phafd_fno_adam_step",
    "phafd_fno_selftest",
]

C_CH = 32          # channels
NKX, NK = 8, 16    # retained kx in [0, 8); ky, kz in [-8, 8)
NMODE = NK * NK * NKX
LSZ = 1024 + 32 + NMODE * C_CH * C_CH * 2


def layout():
    """Offsets of the parameter groups in the flat vector."""
    off = {"P": (0, (32, 16)), "pb": (512, (32,))}
    base = 544
    for l in range(4):
        off["W%d" % l] = (base, (32, 32))
        off["b%d" % l] = (base + 1024, (32,))
        off["R%d" % l] = (base + 1056, (NMODE, 32, 32, 2))
        base += LSZ
    off["Q1"] = (base, (32, 32))
    off["q1b"] = (base + 1024, (32,))
    off["q2"] = (base + 1056, (32,))
    off["q2b"] = (base + 1088, (1,))
    return off


def param_count():
    return 544 + 4 * LSZ + 1089


def unpack(vec):
    """dict of views into a flat parameter vector."""
    out = {}
    for k, (o, shp) in layout().items():
        n = int(np.prod(shp))
        out[k] = vec[o:o + n].reshape(shp)
    return out


def init_params(seed=0, out_scale=0.0):
    """Random initial parameters: uniform(+-1/sqrt(fan_in)) pointwise weights,
    spectral weights uniform in [0, 1/(32*32)) (the usual Fourier-layer
    scale), zero biases, q2 scaled by out_scale (0: the correction starts at 0)."""
    rng = np.random.default_rng(seed)
    v = np.zeros(param_count(), np.float32)
    p = unpack(v)
    p["P"][:, :3] = rng.uniform(-1 / np.sqrt(3), 1 / np.sqrt(3), (32, 3))
    for l in range(4):
        p["W%d" % l][:] = rng.uniform(-1 / np.sqrt(32), 1 / np.sqrt(32), (32, 32))
        p["R%d" % l][:] = rng.uniform(0, 1.0 / (32 * 32), (NMODE, 32, 32, 2))
    p["Q1"][:] = rng.uniform(-1 / np.sqrt(32), 1 / np.sqrt(32), (32, 32))
    p["q2"][:] = out_scale * rng.uniform(-1 / np.sqrt(32), 1 / np.sqrt(32), 32)
    return v


_bound = False


def _lib():
    global _bound
    L = load()
    if not _bound:
        vp = C.c_void_p
        fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.phafd_fno_param_count.argtypes = []
        L.phafd_fno_param_count.restype = C.c_size_t
        sig = {
            "phafd_fno_create": [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int],
            "phafd_fno_destroy": [vp],
            "phafd_fno_set_params": [vp, fp, C.c_size_t],
            "phafd_fno_get_params": [vp, fp, C.c_size_t],
            "phafd_fno_set_norm": [vp, fp],
            "phafd_fno_infer": [vp, vp, vp, C.c_float, vp, vp],
            "phafd_fno_zero_grad": [vp],
            "phafd_fno_forward_backward": [vp, vp, vp, C.c_float, vp, C.POINTER(C.c_double)],
            "phafd_fno_get_grad": [vp, fp, C.c_size_t],
            "phafd_fno_adam_step": [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int],
            "phafd_fno_selftest": [C.c_int, np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")],
        }
        for k, a in sig.items():
            getattr(L, k).argtypes = a
            getattr(L, k).restype = C.c_int
        L.phafd_fno_last_error.argtypes = [vp]
        L.phafd_fno_last_error.restype = C.c_char_p
        _bound = True
    return L


def selftest(device=0):
    """(K-major products exact, MN-major products exact) on this GPU."""
    r = np.zeros(2, np.int32)
    rc = _lib().phafd_fno_selftest(device, r)
    if rc != 0:
        raise RuntimeError("phafd_fno_selftest failed (%s)" % ERRORS.get(rc, rc))
    return bool(r[0]), bool(r[1])


class FNOError(RuntimeError):
    pass


class FNO:
    """The learned propagator for grids of (nz, ny, nx) nodes on one GPU."""

    def __init__(self, shape, device=0, train=False):
        self._L = _lib()
        self._f = C.c_void_p()
        nz, ny, nx = shape
        rc = self._L.phafd_fno_create(C.byref(self._f), device, nx, ny, nz, int(train))
        if rc != 0:
            raise FNOError("phafd_fno_create(%d, %d, %d) failed (%s)" % (nx, ny, nz, ERRORS.get(rc, rc)))
        self.shape = shape
        self.train = train
        self.norm = np.array([0.45, 0.05, 0.0, 1.0, 3.0, 0.3, 1.0, 0.0], np.float32)

    def close(self):
        if getattr(self, "_f", None):
            self._L.phafd_fno_destroy(self._f)
            self._f = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise FNOError("%s: %s (%s)" % (what, self._L.phafd_fno_last_error(self._f).decode(), ERRORS.get(rc, rc)))

    def set_params(self, vec):
        v = np.ascontiguousarray(vec, np.float32)
        self._chk(self._L.phafd_fno_set_params(self._f, v, v.size), "set_params")

    def get_params(self):
        v = np.zeros(param_count(), np.float32)
        self._chk(self._L.phafd_fno_get_params(self._f, v, v.size), "get_params")
        return v

    def set_norm(self, norm):
        self.norm = np.ascontiguousarray(norm, np.float32)
        self._chk(self._L.phafd_fno_set_norm(self._f, self.norm), "set_norm")

    def infer(self, phi_ptr, rho_ptr, chi, corr_ptr, stream=None):
        self._chk(self._L.phafd_fno_infer(self._f, C.c_void_p(phi_ptr), C.c_void_p(rho_ptr), float(chi),
                                          C.c_void_p(corr_ptr), C.c_void_p(stream)), "infer")

    def zero_grad(self):
        self._chk(self._L.phafd_fno_zero_grad(self._f), "zero_grad")

    def forward_backward(self, phi_ptr, rho_ptr, chi, target_ptr):
        loss = C.c_double(0.0)
        self._chk(self._L.phafd_fno_forward_backward(self._f, C.c_void_p(phi_ptr), C.c_void_p(rho_ptr), float(chi),
                                                     C.c_void_p(target_ptr), C.byref(loss)), "forward_backward")
        return loss.value

    def get_grad(self):
        g = np.zeros(param_count(), np.float32)
        self._chk(self._L.phafd_fno_get_grad(self._f, g, g.size), "get_grad")
        return g

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, nbatch=1):
        self._chk(self._L.phafd_fno_adam_step(self._f, float(lr), float(beta1), float(beta2), float(eps), int(nbatch)),
                  "adam_step")

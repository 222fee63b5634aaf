"""ctypes wrapper of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module, and only as the checker.  The method names match
phafd_gb300.PhafdGPU so that a test drives both with one call sequence.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

FIELD = {"phi": 0, "chempot": 1, "gradx": 2, "grady": 3, "gradz": 4, "ft_phi": 5, "ft_chempot": 6}
GRIDATOM = {"none": 0, "gaussian": 1, "LJish": 2, "LJish/linear": 3}
NOISE = {"off": 0, "reference": 1, "philox": 2}
ZGHOST = {"rank1": 0, "periodic": 1}
PAIR = {"lj/cut": 1, "gridatom": 2}


class SemiParams(C.Structure):
    _fields_ = [("bondlength", C.c_double), ("zeta_para", C.c_double), ("zeta_perp", C.c_double),
                ("bending", C.c_double), ("temp", C.c_double), ("kbond", C.c_double),
                ("seed", C.c_int), ("noise", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        vp = C.c_void_p
        sig = {
            "oracle_ctx_create": [C.POINTER(vp)],
            "oracle_last_error": [vp],
            "oracle_set_zghost": [vp, C.c_int],
            "oracle_domain": [vp, dp, dp],
            "oracle_grid_style": [vp, C.c_int, C.c_int, C.c_int],
            "oracle_grid_populate_constant": [vp, C.c_double, C.c_double, C.c_int],
            "oracle_grid_populate_flat_interface": [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int],
            "oracle_grid_populate_sphere": [vp, C.c_double, C.c_double, C.c_double, C.c_double],
            "oracle_grid_set": [vp, C.c_int, dp],
            "oracle_grid_get": [vp, C.c_int, dp],
            "oracle_atoms_create": [vp, C.c_int, ip, ip, ip, dp],
            "oracle_atoms_get": [vp, dp, dp, dp, ip],
            "oracle_atoms_set_images": [vp, ip],
            "oracle_pair_gridatom": [vp, C.c_int, C.c_double],
            "oracle_pair_gridatom_coeff": [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double],
            "oracle_pair_lj_cut": [vp, C.c_double, C.c_double, C.c_double],
            "oracle_neighbor": [vp, C.c_double],
            "oracle_fix_conjugate_volfrac": [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int],
            "oracle_fix_floryhuggins": [vp, C.c_double, C.c_double, C.c_double],
            "oracle_fix_gradphi": [vp, C.c_int],
            "oracle_fix_drag": [vp, C.c_int, ip, ip, C.c_double],
            "oracle_fix_semiflexible": [vp, C.c_int, ip, ip, C.POINTER(SemiParams)],
            "oracle_set_dt": [vp, C.c_double],
            "oracle_set_timestep": [vp, C.c_longlong],
            "oracle_setup": [vp],
            "oracle_run": [vp, C.c_int],
            "oracle_compute_grid_clusters": [vp, C.c_double, C.c_int,
                                             np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")],
            "oracle_run_until_touching": [vp, C.c_longlong, C.c_double, C.c_int, C.c_int,
                                          C.POINTER(C.c_longlong), C.c_int,
                                          np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS"),
                                          np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"),
                                          C.POINTER(C.c_int)],
            "oracle_compute_pair": [vp, C.c_int, dp],
            "oracle_stage_gradient": [vp],
            "oracle_stage_borders_and_build": [vp],
            "oracle_stage_pairs": [vp],
            "oracle_half_list_size": [vp],
            "oracle_grid_list_size": [vp],
            "oracle_half_list": [vp, ip],
            "oracle_grid_list": [vp, ip],
            "oracle_counters": [vp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")],
            "oracle_stage_times": [vp, dp],
            "oracle_fft_r2c": [C.c_int, C.c_int, C.c_int, dp, dp],
            "oracle_fft_c2r": [C.c_int, C.c_int, C.c_int, dp, dp],
            "oracle_make_unique_seed": [C.c_int],
            "oracle_set_threads": [C.c_int],
            "oracle_noise_state_get": [vp, C.c_char_p, C.c_int, C.POINTER(C.c_int)],
            "oracle_noise_state_set": [vp, C.c_char_p],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_ctx_destroy.argtypes = [vp]
        L.oracle_ctx_destroy.restype = None
        L.oracle_chain_force.argtypes = [dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]
        L.oracle_chain_force.restype = None
        L.oracle_bead_gauss.argtypes = [C.c_uint32, C.c_uint64, C.c_int, C.c_int, dp]
        L.oracle_bead_gauss.restype = None
        _lib = L
    return _lib


def set_threads(n):
    """Host threads of the oracle's grid loops (FFT lines, pointwise passes,
    the bulk mode update).  Results are bit-identical for any count."""
    lib().oracle_set_threads(int(n))


def host_threads():
    """The cores this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def fft_r2c(phi):
    """FFTW-convention r2c of a real [z][y][x] array, returned in the
    reference's transposed k-space layout [ky][kz][kx]."""
    nz, ny, nx = phi.shape
    out = np.zeros((ny, nz, nx // 2 + 1), dtype=np.complex128)
    rc = lib().oracle_fft_r2c(nx, ny, nz, np.ascontiguousarray(phi, dtype=np.float64), out.view(np.float64).reshape(-1))
    assert rc == 0
    return out


def fft_c2r(spec, shape):
    nz, ny, nx = shape
    out = np.zeros(shape, dtype=np.float64)
    rc = lib().oracle_fft_c2r(nx, ny, nz, np.ascontiguousarray(spec).view(np.float64).reshape(-1), out.reshape(-1))
    assert rc == 0
    return out


def make_unique_seed(seed):
    return lib().oracle_make_unique_seed(int(seed))


def bead_gauss(seed, step, half, bead):
    out = np.zeros(3)
    lib().oracle_bead_gauss(seed, step, half, bead, out)
    return out


class OracleError(RuntimeError):
    pass


class Oracle:
    """FP64 CPU restatement of the reference's one-rank timestep."""

    def __init__(self):
        self._L = lib()
        self._c = C.c_void_p()
        self._call("oracle_ctx_create", C.byref(self._c), ctx=False)
        self.shape = None
        self.n = 0

    def __del__(self):
        try:
            if self._c:
                self._L.oracle_ctx_destroy(self._c)
                self._c = C.c_void_p()
        except Exception:
            pass

    def _call(self, name, *args, ctx=True):
        f = getattr(self._L, name)
        rc = f(self._c, *args) if ctx else f(*args)
        if rc != 0:
            msg = self._L.oracle_last_error(self._c).decode() if self._c else name
            raise OracleError(msg)
        return rc

    # ---- set-up commands
    def set_zghost(self, mode):
        self._call("oracle_set_zghost", ZGHOST[mode])

    def domain(self, boxlo, period):
        self._call("oracle_domain", np.asarray(boxlo, np.float64), np.asarray(period, np.float64))

    def grid_style(self, nx, ny, nz):
        self._call("oracle_grid_style", nx, ny, nz)
        self.shape = (nz, ny, nx)

    def grid_populate_constant(self, average, variance, seed):
        self._call("oracle_grid_populate_constant", average, variance, seed)

    def grid_populate_flat_interface(self, average, variance, hi, lo, seed):
        self._call("oracle_grid_populate_flat_interface", average, variance, hi, lo, seed)

    def grid_populate_sphere(self, radius, width, hi, average):
        self._call("oracle_grid_populate_sphere", radius, width, hi, average)

    def grid_set(self, field, arr):
        self._call("oracle_grid_set", FIELD[field], np.ascontiguousarray(arr, np.float64).reshape(-1))

    def grid_get(self, field):
        nz, ny, nx = self.shape
        if field.startswith("ft_"):
            out = np.zeros((ny, nz, nx // 2 + 1), np.complex128)
            self._call("oracle_grid_get", FIELD[field], out.view(np.float64).reshape(-1))
        else:
            out = np.zeros(self.shape, np.float64)
            self._call("oracle_grid_get", FIELD[field], out.reshape(-1))
        return out

    def atoms_create(self, tags, mol, types, x):
        self.n = len(tags)
        self._call("oracle_atoms_create", self.n, np.asarray(tags, np.int32), np.asarray(mol, np.int32),
                   np.asarray(types, np.int32), np.ascontiguousarray(x, np.float64).reshape(-1))

    def noise_state(self):
        """the reference-noise generator's state (text)"""
        n = C.c_int(0)
        self._call("oracle_noise_state_get", None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        self._call("oracle_noise_state_get", buf, n.value, C.byref(n))
        return buf.value.decode()

    def set_noise_state(self, state):
        self._call("oracle_noise_state_set", state.encode())

    def atoms_set_images(self, images):
        im = np.ascontiguousarray(images, np.int32)
        if len(im) != self.n:
            raise ValueError("one image flag per bead")
        self._call("oracle_atoms_set_images", np.ascontiguousarray(np.resize(im, max(self.n, 1))))

    def atoms_get(self):
        x = np.zeros((self.n, 3)); ux = np.zeros((self.n, 3)); f = np.zeros((self.n, 3))
        im = np.zeros(self.n, np.int32)
        self._call("oracle_atoms_get", x.reshape(-1), ux.reshape(-1), f.reshape(-1), im)
        return x, ux, f, im

    def pair_gridatom(self, style, cut):
        self._call("oracle_pair_gridatom", GRIDATOM[style], cut)

    def pair_gridatom_coeff(self, t, epsilon=None, nucwidth=None, phi=None):
        self._call("oracle_pair_gridatom_coeff", t, epsilon is not None, epsilon or 0.0,
                   nucwidth is not None, nucwidth or 0.0, phi is not None, phi or 0.0)

    def pair_lj_cut(self, cut, eps, sigma):
        self._call("oracle_pair_lj_cut", cut, eps, sigma)

    def neighbor(self, skin):
        self._call("oracle_neighbor", skin)

    def fix_conjugate_volfrac(self, seed, mobility=1.0, temp=1.0, volFH=1.0, gamma=1.0, noise="reference"):
        self._call("oracle_fix_conjugate_volfrac", seed, mobility, temp, volFH, gamma, NOISE[noise])

    def fix_floryhuggins(self, temp=1.0, volFH=1.0, chi=1.0):
        self._call("oracle_fix_floryhuggins", temp, volFH, chi)

    def fix_gradphi(self, once=False):
        self._call("oracle_fix_gradphi", int(once))

    def fix_drag(self, ranges, drag):
        s = np.array([r[0] for r in ranges], np.int32); e = np.array([r[1] for r in ranges], np.int32)
        self._call("oracle_fix_drag", len(ranges), s, e, drag)

    def fix_semiflexible(self, ranges, bondlength=1.0, zeta_para=1.0, zeta_perp=1.0, bending=0.0,
                         temp=0.0, kbond=100.0, seed=0, noise="philox"):
        s = np.array([r[0] for r in ranges], np.int32); e = np.array([r[1] for r in ranges], np.int32)
        p = SemiParams(bondlength, zeta_para, zeta_perp, bending, temp, kbond, seed, NOISE[noise])
        self._call("oracle_fix_semiflexible", len(ranges), s, e, C.byref(p))

    def set_dt(self, dt):
        self._call("oracle_set_dt", dt)

    def set_timestep(self, ts):
        self._call("oracle_set_timestep", ts)

    def setup(self):
        self._call("oracle_setup")

    def run(self, nsteps):
        self._call("oracle_run", nsteps)

    def run_until_touching(self, nsteps, touch_point, continue_running=False, delay_step=0, max_events=1024):
        """Integrate::run_until_touching (integrate.cpp:221-415): (steps run,
        [(kind, step)]) with kind 0 = cyclisation at step, 1 = interval ended."""
        done = C.c_longlong(0)
        nev = C.c_int(0)
        steps = np.zeros(max_events, np.int64)
        kinds = np.zeros(max_events, np.int32)
        self._call("oracle_run_until_touching", int(nsteps), float(touch_point), int(bool(continue_running)),
                   int(delay_step), C.byref(done), int(max_events), steps, kinds, C.byref(nev))
        k = min(nev.value, max_events)
        return done.value, list(zip(kinds[:k].tolist(), steps[:k].tolist()))

    def compute_grid_clusters(self, threshold, condition="gt"):
        """Labels of compute grid/cluster (compute_grid_clusters.cpp:66-229):
        int32 [z][y][x], -1 outside the clusters."""
        if condition not in ("lt", "gt"):
            raise ValueError("Must specify lt or gt for compute grid cluster.")
        out = np.zeros(self.shape, np.int32)
        self._call("oracle_compute_grid_clusters", float(threshold), int(condition == "gt"), out)
        return out

    # ---- stage hooks and inspection
    def compute_pair(self, style, add_to_chempot=True):
        """compute pair (compute_pair.cpp:43-85) after the last step: forces of
        "lj/cut" or "gridatom" per owned bead, (n, 3); the style's chempot
        deposit lands in chempot as in the reference (add_to_chempot is the
        GPU library's switch for the same side effect; the oracle always
        follows the reference)."""
        n = self.atoms_get()[0].shape[0]
        out = np.zeros((n, 3))
        self._call("oracle_compute_pair", PAIR[style], out)
        return out

    def stage_gradient(self):
        self._call("oracle_stage_gradient")

    def stage_borders_and_build(self):
        self._call("oracle_stage_borders_and_build")

    def stage_pairs(self):
        self._call("oracle_stage_pairs")

    def half_list(self):
        n = self._L.oracle_half_list_size(self._c)
        out = np.zeros(3 * n, np.int32)
        self._call("oracle_half_list", out)
        return out.reshape(n, 3)

    def grid_list(self):
        n = self._L.oracle_grid_list_size(self._c)
        out = np.zeros(3 * n, np.int32)
        self._call("oracle_grid_list", out)
        return out.reshape(n, 3)

    def counters(self):
        out = np.zeros(6, np.int64)
        self._call("oracle_counters", out)
        return dict(num_less_zero=int(out[0]), num_great_zero=int(out[1]), neighbor_calls=int(out[2]),
                    timestep=int(out[3]), nlocal=int(out[4]), nghost=int(out[5]))

    def stage_times(self):
        out = np.zeros(7)
        self._call("oracle_stage_times", out)
        return out

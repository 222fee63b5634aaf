"""ctypes binding of libphafd_gpu.so (the C ABI in include/phafd_gpu.h).

`PhafdGPU` mirrors the reference's input-script commands one method per
command (input.cpp:48-299).  There is no CPU fallback: if the library is
missing or fails to load, construction raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libphafd_gpu.so")

FIELD = {"phi": 0, "chempot": 1, "gradx": 2, "grady": 3, "gradz": 4, "ft_phi": 5, "ft_chempot": 6,
         "ft_phi_step_start": 7, "gradx_step_start": 8, "grady_step_start": 9, "gradz_step_start": 10}
PAIR = {"lj/cut": 1, "gridatom": 2}
GRIDATOM = {"none": 0, "gaussian": 1, "LJish": 2, "LJish/linear": 3}
NOISE = {"off": 0, "reference": 1, "philox": 2}
ZGHOST = {"rank1": 0, "periodic": 1}
SCHEDULE = {"reference": 0, "resident": 1}
ERRORS = {-1: "invalid", -2: "cuda", -3: "nan", -4: "overflow", -5: "constraint", -6: "unsupported", -7: "nomem",
          -8: "timeout"}

# every symbol declared in include/phafd_gpu.h
EXPORTS = [
    "phafd_ctx_create", "phafd_ctx_destroy", "phafd_last_error", "phafd_build_info",
    "phafd_domain", "phafd_grid_style", "phafd_grid_populate_constant", "phafd_grid_populate_flat_interface",
    "phafd_grid_populate_sphere", "phafd_grid_set", "phafd_grid_get",
    "phafd_set_zghost", "phafd_set_schedule", "phafd_set_keep_chempot", "phafd_set_plane_fusion",
    "phafd_set_gradient_mask", "phafd_set_fp32_centering", "phafd_set_pair_snapshot", "phafd_compute_pair",
    "phafd_set_variants", "phafd_autotune", "phafd_set_graph_steps",
    "phafd_atoms_create", "phafd_atoms_get", "phafd_atoms_set_images", "phafd_atoms_get_async", "phafd_wait_slot",
    "phafd_host_register", "phafd_host_unregister",
    "phafd_pair_gridatom", "phafd_pair_gridatom_coeff", "phafd_pair_lj_cut",
    "phafd_neighbor",
    "phafd_fix_conjugate_volfrac", "phafd_fix_floryhuggins", "phafd_fix_gradphi", "phafd_fix_drag",
    "phafd_fix_semiflexible",
    "phafd_set_dt", "phafd_set_timestep", "phafd_noise_state_get", "phafd_noise_state_set", "phafd_setup", "phafd_run", "phafd_run_async", "phafd_counters_get",
    "phafd_synchronize",
    "phafd_run_timed", "phafd_profile_stages",
    "phafd_half_list_size", "phafd_half_list", "phafd_grid_list_size", "phafd_grid_list",
    "phafd_stage_gradient", "phafd_stage_borders_and_build", "phafd_stage_pairs",
    "phafd_gradphi_noalloc",
    "phafd_compute_complex", "phafd_structure_factor", "phafd_compute_grid_clusters", "phafd_run_until_touching",
    "phafd_set_linear_substeps", "phafd_grid_device", "phafd_grid_copy_device", "phafd_deposit_density",
    "phafd_grid_add_device", "phafd_ctx_copy_state",
]


class SemiParams(C.Structure):
    _fields_ = [("bondlength", C.c_double), ("zeta_para", C.c_double), ("zeta_perp", C.c_double),
                ("bending", C.c_double), ("temp", C.c_double), ("kbond", C.c_double),
                ("seed", C.c_int), ("noise", C.c_int)]


class Counters(C.Structure):
    _fields_ = [("num_less_zero", C.c_longlong), ("num_great_zero", C.c_longlong),
                ("neighbor_calls", C.c_longlong), ("timestep", C.c_longlong),
                ("status", C.c_longlong), ("nan_step", C.c_longlong), ("kernels_per_step", C.c_longlong),
                ("kernels_per_rebuild", C.c_longlong)]


class PhafdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%s)" % (msg, ERRORS.get(code, code)))
        self.code = code


_lib = None


def load(path=None):
    """Load libphafd_gpu.so; raise if it is absent (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libphafd_gpu.so not built: run __graft_entry__.build() (expected %s)" % p)
    L = C.CDLL(p)
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    vp = C.c_void_p
    sig = {
        "phafd_ctx_create": [C.POINTER(vp), C.c_int, C.c_int],
        "phafd_ctx_destroy": [vp],
        "phafd_set_zghost": [vp, C.c_int],
        "phafd_set_schedule": [vp, C.c_int],
        "phafd_set_keep_chempot": [vp, C.c_int],
        "phafd_set_plane_fusion": [vp, C.c_int],
        "phafd_set_gradient_mask": [vp, C.c_int],
        "phafd_set_fp32_centering": [vp, C.c_int],
        "phafd_set_pair_snapshot": [vp, C.c_int],
        "phafd_set_variants": [vp, C.c_int],
        "phafd_set_graph_steps": [vp, C.c_int],
        "phafd_autotune": [vp, C.c_int, C.POINTER(C.c_int), dp],
        "phafd_compute_pair": [vp, C.c_int, C.c_int, dp],
        "phafd_domain": [vp, dp, dp],
        "phafd_grid_style": [vp, C.c_int, C.c_int, C.c_int],
        "phafd_grid_populate_constant": [vp, C.c_double, C.c_double, C.c_int],
        "phafd_grid_populate_flat_interface": [vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int],
        "phafd_grid_populate_sphere": [vp, C.c_double, C.c_double, C.c_double, C.c_double],
        "phafd_grid_set": [vp, C.c_int, dp],
        "phafd_grid_get": [vp, C.c_int, dp],
        "phafd_atoms_create": [vp, C.c_int, ip, ip, ip, dp],
        "phafd_atoms_get": [vp, dp, dp, dp, ip],
        "phafd_atoms_get_async": [vp, dp, dp, dp, ip, C.c_int],
        "phafd_wait_slot": [vp, C.c_int],
        "phafd_host_register": [C.c_void_p, C.c_size_t],
        "phafd_host_unregister": [C.c_void_p],
        "phafd_atoms_set_images": [vp, ip],
        "phafd_pair_gridatom": [vp, C.c_int, C.c_double],
        "phafd_pair_gridatom_coeff": [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double],
        "phafd_pair_lj_cut": [vp, C.c_double, C.c_double, C.c_double],
        "phafd_neighbor": [vp, C.c_double],
        "phafd_fix_conjugate_volfrac": [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int],
        "phafd_fix_floryhuggins": [vp, C.c_double, C.c_double, C.c_double],
        "phafd_fix_gradphi": [vp, C.c_int],
        "phafd_fix_drag": [vp, C.c_int, ip, ip, C.c_double],
        "phafd_fix_semiflexible": [vp, C.c_int, ip, ip, C.POINTER(SemiParams)],
        "phafd_set_dt": [vp, C.c_double],
        "phafd_set_timestep": [vp, C.c_longlong],
        "phafd_noise_state_get": [vp, C.c_char_p, C.c_int, C.POINTER(C.c_int)],
        "phafd_noise_state_set": [vp, C.c_char_p],
        "phafd_setup": [vp],
        "phafd_run": [vp, C.c_int],
        "phafd_run_async": [vp, C.c_int],
        "phafd_counters_get": [vp, C.POINTER(Counters)],
        "phafd_synchronize": [vp],
        "phafd_run_timed": [vp, C.c_int, C.POINTER(C.c_double)],
        "phafd_profile_stages": [vp, C.c_int, dp, C.c_int],
        "phafd_half_list_size": [vp, C.POINTER(C.c_longlong)],
        "phafd_half_list": [vp, ip],
        "phafd_grid_list_size": [vp, C.POINTER(C.c_longlong)],
        "phafd_grid_list": [vp, ip],
        "phafd_stage_gradient": [vp],
        "phafd_stage_borders_and_build": [vp],
        "phafd_stage_pairs": [vp],
        "phafd_compute_complex": [vp, C.c_int, C.c_int, dp],
        "phafd_structure_factor": [vp, C.c_int, dp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")],
        "phafd_compute_grid_clusters": [vp, C.c_double, C.c_int, C.c_void_p, C.POINTER(C.c_int)],
        "phafd_run_until_touching": [vp, C.c_longlong, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_longlong),
                                     C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)],
        "phafd_set_linear_substeps": [vp, C.c_int, C.c_double],
        "phafd_grid_device": [vp, C.c_int, C.POINTER(vp)],
        "phafd_grid_copy_device": [vp, C.c_int, vp],
        "phafd_deposit_density": [vp, vp],
        "phafd_grid_add_device": [vp, vp, C.c_double],
        "phafd_ctx_copy_state": [vp, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.phafd_last_error.argtypes = [vp]
    L.phafd_last_error.restype = C.c_char_p
    L.phafd_build_info.argtypes = []
    L.phafd_build_info.restype = C.c_char_p
    L.phafd_gradphi_noalloc.argtypes = [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, dp, vp]
    L.phafd_gradphi_noalloc.restype = C.c_int
    _lib = L
    return L


class PhafdGPU:
    """One simulation context on one GPU.  precision: 32 or 64."""

    def __init__(self, precision=64, device=0, schedule="resident"):
        self._L = load()
        self._c = C.c_void_p()
        rc = self._L.phafd_ctx_create(C.byref(self._c), device, precision)
        if rc != 0:
            raise PhafdError(rc, "phafd_ctx_create failed (device %d)" % device)
        self.precision = precision
        self.shape = None
        self.n = 0
        self.set_schedule(schedule)

    def close(self):
        if getattr(self, "_c", None):
            self._L.phafd_ctx_destroy(self._c)
            self._c = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        rc = getattr(self._L, name)(self._c, *args)
        if rc != 0:
            raise PhafdError(rc, self._L.phafd_last_error(self._c).decode())
        return rc

    # ---- commands
    def set_zghost(self, mode):
        self._call("phafd_set_zghost", ZGHOST[mode])

    def set_schedule(self, schedule):
        self._call("phafd_set_schedule", SCHEDULE[schedule])

    def set_keep_chempot(self, keep=True):
        self._call("phafd_set_keep_chempot", int(keep))

    def set_plane_fusion(self, on=True):
        self._call("phafd_set_plane_fusion", int(on))

    def set_gradient_mask(self, on=True):
        """Store grad phi only near the beads during steps (off by default)."""
        self._call("phafd_set_gradient_mask", int(on))

    def set_variants(self, plane=False, generic256=False, xc2r_tma=True, xr2c_tma=True):
        """Kernel variants of the step (PHAFD_TUNE_*; a new context has
        xc2r_tma and xr2c_tma on)."""
        self._call("phafd_set_variants", (1 if plane else 0) | (2 if generic256 else 0) | (4 if xc2r_tma else 0)
                   | (8 if xr2c_tma else 0))

    def set_graph_steps(self, steps):
        """Steps per CUDA graph of a run (even, >= 2; default 8)."""
        self._call("phafd_set_graph_steps", steps)

    def autotune(self, steps=10):
        """Time every variant over `steps` steps of the run, keep the fastest:
        returns (best flags, ms per step by flags, -1 where not applicable)."""
        best = C.c_int(0)
        ms = np.zeros(16)
        self._call("phafd_autotune", steps, C.byref(best), ms)
        return best.value, ms

    def set_pair_snapshot(self, on=True):
        """Keep each step's pair-stage positions (needed by compute_pair)."""
        self._call("phafd_set_pair_snapshot", int(on))

    def compute_pair(self, style, add_to_chempot=True):
        """compute pair after the last step: forces of "lj/cut" or "gridatom"
        per bead, (n, 3) (compute_pair.cpp:43-85)."""
        out = np.zeros((max(self.n, 1), 3))
        self._call("phafd_compute_pair", PAIR[style], int(add_to_chempot), out)
        return out[:self.n]

    def set_fp32_centering(self, fh=False, fft=True):
        """FP32 stages taken relative to the mean of phi (the transforms by default)."""
        self._call("phafd_set_fp32_centering", (1 if fh else 0) | (2 if fft else 0))

    def domain(self, boxlo, period):
        self._call("phafd_domain", np.asarray(boxlo, np.float64), np.asarray(period, np.float64))

    def grid_style(self, nx, ny, nz):
        self._call("phafd_grid_style", nx, ny, nz)
        self.shape = (nz, ny, nx)

    def grid_populate_constant(self, average, variance, seed):
        self._call("phafd_grid_populate_constant", average, variance, seed)

    def grid_populate_flat_interface(self, average, variance, hi, lo, seed):
        self._call("phafd_grid_populate_flat_interface", average, variance, hi, lo, seed)

    def grid_populate_sphere(self, radius, width, hi, average):
        self._call("phafd_grid_populate_sphere", radius, width, hi, average)

    def grid_set(self, field, arr):
        self._call("phafd_grid_set", FIELD[field], np.ascontiguousarray(arr, np.float64).reshape(-1))

    def grid_get(self, field):
        nz, ny, nx = self.shape
        if field.startswith("ft_"):
            out = np.zeros((ny, nz, nx // 2 + 1), np.complex128)
            self._call("phafd_grid_get", FIELD[field], out.view(np.float64).reshape(-1))
        else:
            out = np.zeros(self.shape, np.float64)
            self._call("phafd_grid_get", FIELD[field], out.reshape(-1))
        return out

    # ---- spectra and the learned macro step
    COMPLEX = {"real": 0, "imag": 1, "modulus": 2, "norm": 3}

    def compute_complex(self, field, quant):
        """compute complex ft_phi|ft_chempot real|imag|modulus|norm, layout [ky][kz][kx]."""
        nz, ny, nx = self.shape
        out = np.zeros((ny, nz, nx // 2 + 1), np.float64)
        self._call("phafd_compute_complex", FIELD[field], self.COMPLEX[quant], out.reshape(-1))
        return out

    def run_until_touching(self, nsteps, touch_point, continue_running=False, delay_step=0, max_events=1024):
        """Integrate::run_until_touching: (steps run, [(kind, step)]), kind 0 =
        cyclisation at step, 1 = cyclisation interval ended at step."""
        done = C.c_longlong(0)
        nev = C.c_int(0)
        steps = np.zeros(max_events, np.int64)
        kinds = np.zeros(max_events, np.int32)
        self._call("phafd_run_until_touching", int(nsteps), float(touch_point), int(bool(continue_running)),
                   int(delay_step), C.byref(done), int(max_events), steps.ctypes.data_as(C.c_void_p),
                   kinds.ctypes.data_as(C.c_void_p), C.byref(nev))
        k = min(nev.value, max_events)
        return done.value, list(zip(kinds[:k].tolist(), steps[:k].tolist()))

    def compute_grid_clusters(self, threshold, condition="gt"):
        """compute grid/cluster phi threshold gt|lt: (labels int32 [z][y][x],
        -1 outside the clusters; number of clusters)."""
        if condition not in ("lt", "gt"):
            raise ValueError("Must specify lt or gt for compute grid cluster.")
        out = np.zeros(self.shape, np.int32)
        ncl = C.c_int(0)
        self._call("phafd_compute_grid_clusters", float(threshold), int(condition == "gt"),
                   out.ctypes.data_as(C.c_void_p), C.byref(ncl))
        return out, ncl.value

    def structure_factor(self, nbins):
        sk = np.zeros(nbins, np.float64)
        cnt = np.zeros(nbins, np.int64)
        self._call("phafd_structure_factor", nbins, sk, cnt)
        return sk, cnt

    def set_linear_substeps(self, nsub, f2=0.0):
        self._call("phafd_set_linear_substeps", int(nsub), float(f2))

    def grid_device(self, field="phi"):
        p = C.c_void_p()
        self._call("phafd_grid_device", FIELD[field], C.byref(p))
        return p.value

    def grid_copy_device(self, field, dst_ptr):
        """Copy a real field into the device array at dst_ptr (waits for it)."""
        self._call("phafd_grid_copy_device", FIELD[field], C.c_void_p(dst_ptr))

    def deposit_density(self, rho_ptr):
        self._call("phafd_deposit_density", C.c_void_p(rho_ptr))

    def grid_add_device(self, src_ptr, scale=1.0):
        self._call("phafd_grid_add_device", C.c_void_p(src_ptr), float(scale))

    def copy_state_from(self, other):
        """this context's dynamic state := other's (same set-up)."""
        self._call("phafd_ctx_copy_state", other._c)

    def atoms_create(self, tags, mol, types, x):
        self.n = len(tags)
        self._call("phafd_atoms_create", self.n, np.asarray(tags, np.int32), np.asarray(mol, np.int32),
                   np.asarray(types, np.int32), np.ascontiguousarray(x, np.float64).reshape(-1))

    def atoms_get(self):
        n = max(self.n, 1)
        x = np.zeros((n, 3)); ux = np.zeros((n, 3)); f = np.zeros((n, 3)); im = np.zeros(n, np.int32)
        self._call("phafd_atoms_get", x.reshape(-1), ux.reshape(-1), f.reshape(-1), im)
        return x[:self.n], ux[:self.n], f[:self.n], im[:self.n]

    def atoms_get_async(self, bufs, slot):
        """Enqueue the beads' read-back (x, ux, F, image flags) into the
        caller's arrays bufs = (x, ux, f, images), which must stay alive until
        wait_slot(slot); page-locked (host_register) they fill while later
        steps compute."""
        x, ux, f, im = bufs
        self._call("phafd_atoms_get_async", x.reshape(-1), ux.reshape(-1), f.reshape(-1), im, slot)

    def wait_slot(self, slot):
        """Wait for the read-back enqueued on `slot`; raise on a device error."""
        self._call("phafd_wait_slot", slot)

    def noise_state(self):
        """the reference-noise generator's state (text), for a restart"""
        n = C.c_int(0)
        self._call("phafd_noise_state_get", None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value)
        self._call("phafd_noise_state_get", buf, n.value, C.byref(n))
        return buf.value.decode()

    def set_noise_state(self, state):
        self._call("phafd_noise_state_set", state.encode())

    def atoms_set_images(self, images):
        """packed image flags of every bead (restart), before setup."""
        im = np.ascontiguousarray(images, np.int32)
        if len(im) != self.n:
            raise ValueError("one image flag per bead")
        self._call("phafd_atoms_set_images", np.ascontiguousarray(np.resize(im, max(self.n, 1))))

    def pair_gridatom(self, style, cut):
        self._call("phafd_pair_gridatom", GRIDATOM[style], cut)

    def pair_gridatom_coeff(self, t, epsilon=None, nucwidth=None, phi=None):
        self._call("phafd_pair_gridatom_coeff", t, epsilon is not None, epsilon or 0.0,
                   nucwidth is not None, nucwidth or 0.0, phi is not None, phi or 0.0)

    def pair_lj_cut(self, cut, eps, sigma):
        self._call("phafd_pair_lj_cut", cut, eps, sigma)

    def neighbor(self, skin):
        self._call("phafd_neighbor", skin)

    def fix_conjugate_volfrac(self, seed, mobility=1.0, temp=1.0, volFH=1.0, gamma=1.0, noise="philox"):
        self._call("phafd_fix_conjugate_volfrac", seed, mobility, temp, volFH, gamma, NOISE[noise])

    def fix_floryhuggins(self, temp=1.0, volFH=1.0, chi=1.0):
        self._call("phafd_fix_floryhuggins", temp, volFH, chi)

    def fix_gradphi(self, once=False):
        self._call("phafd_fix_gradphi", int(once))

    def fix_drag(self, ranges, drag):
        s = np.array([r[0] for r in ranges], np.int32); e = np.array([r[1] for r in ranges], np.int32)
        self._call("phafd_fix_drag", len(ranges), s, e, drag)

    def fix_semiflexible(self, ranges, bondlength=1.0, zeta_para=1.0, zeta_perp=1.0, bending=0.0,
                         temp=0.0, kbond=100.0, seed=0, noise="philox"):
        s = np.array([r[0] for r in ranges], np.int32); e = np.array([r[1] for r in ranges], np.int32)
        p = SemiParams(bondlength, zeta_para, zeta_perp, bending, temp, kbond, seed, NOISE[noise])
        self._call("phafd_fix_semiflexible", len(ranges), s, e, C.byref(p))

    def set_dt(self, dt):
        self._call("phafd_set_dt", dt)

    def set_timestep(self, ts):
        self._call("phafd_set_timestep", ts)

    def setup(self):
        self._call("phafd_setup")

    def run(self, nsteps):
        self._call("phafd_run", nsteps)

    def run_async(self, nsteps):
        """Enqueue `nsteps` steps and return; synchronize() waits and raises on
        a device-side failure."""
        self._call("phafd_run_async", nsteps)

    def synchronize(self):
        self._call("phafd_synchronize")

    def run_timed(self, nsteps):
        """Run `nsteps` steps; return device milliseconds (CUDA events on
        the library's stream)."""
        ms = C.c_double()
        self._call("phafd_run_timed", nsteps, C.byref(ms))
        return ms.value

    # stage 6 is the z fft of mu in the reference schedule; the resident one
    # fuses its z fft into stage 7 (its stage 6 is empty)
    STAGES = ["gradient", "neighbor", "pairs", "bead_integrate", "x_r2c_fh", "y_fft", "z_fft",
              "z_update_ifft", "y_ifft", "x_c2r"]

    def profile_stages(self, nsteps):
        out = np.zeros(len(self.STAGES))
        self._call("phafd_profile_stages", nsteps, out, len(out))
        return dict(zip(self.STAGES, (out / nsteps).tolist()))

    def counters(self):
        c = Counters()
        self._call("phafd_counters_get", C.byref(c))
        return {k: getattr(c, k) for k, _ in Counters._fields_}

    # ---- stage hooks / inspection
    def stage_gradient(self):
        self._call("phafd_stage_gradient")

    def stage_borders_and_build(self):
        self._call("phafd_stage_borders_and_build")

    def stage_pairs(self):
        self._call("phafd_stage_pairs")

    def half_list(self):
        n = C.c_longlong()
        self._call("phafd_half_list_size", C.byref(n))
        out = np.zeros(3 * max(n.value, 1), np.int32)
        self._call("phafd_half_list", out)
        return out[:3 * n.value].reshape(n.value, 3)

    def grid_list(self):
        n = C.c_longlong()
        self._call("phafd_grid_list_size", C.byref(n))
        out = np.zeros(3 * max(n.value, 1), np.int32)
        self._call("phafd_grid_list", out)
        return out[:3 * n.value].reshape(n.value, 3)


def host_register(arr):
    """Page-lock a numpy array's memory for asynchronous copies."""
    rc = load().phafd_host_register(arr.ctypes.data, arr.nbytes)
    if rc:
        raise PhafdError(rc, "cudaHostRegister failed")


def host_unregister(arr):
    load().phafd_host_unregister(arr.ctypes.data)


def build_info():
    return load().phafd_build_info().decode()

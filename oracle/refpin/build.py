"""Build recipe of oracle/_ref/phafd_ref: the reference's own sources, compiled
unmodified from where they lie (the reference checkout's src/ directory) against
the project-written stand-ins of their absent third-party libraries
(include/: one-rank MPI, FFTW-MPI plans over a project DFT, the Eigen subset
the sources use, fftw_arr's array3D, a beadrodpmer that refuses to run), plus
driver.cpp in place of the reference's main.cpp.

Test infrastructure only: the program generates the reference fixtures under
tests/golden/ that pin the oracle.  Nothing in the product builds or runs it.
The reference's sources are not copied into this repository; the build reads
them in place (PHAFD_REFERENCE_SRC overrides their location) and writes only
under oracle/_ref/.  Where the sources are absent (on a machine without the
reference checkout) build() returns None.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
OBJ = os.path.join(OUT, "obj")
EXE = os.path.join(OUT, "phafd_ref")
REF_SRC = os.environ.get("PHAFD_REFERENCE_SRC", "/root/reference/src")

# the reference's executable (its CMakeLists.txt), main.cpp replaced by the driver
SOURCES = [
    "phafd.cpp", "atom.cpp", "domain.cpp", "grid.cpp", "comm_brick.cpp", "neighbor.cpp", "group.cpp", "input.cpp",
    "nbin.cpp", "nbin_standard.cpp", "neigh_list.cpp", "npair.cpp", "npair_grid_bin.cpp", "npair_half_bin_newton.cpp",
    "nstencil.cpp", "nstencil_full_bin_3d.cpp", "nstencil_half_bin_3d.cpp", "my_page.cpp", "utility.cpp",
    "read_atoms.cpp", "fix.cpp", "fixatom_semiflexible.cpp", "fixgrid_conjugate.cpp", "pair.cpp",
    "pair_gridatom_gaussian.cpp", "pair_gridatom_lj_ish.cpp", "pair_lj_cut.cpp", "pair_harmonic_cut.cpp",
    "fixgrid_floryhuggins.cpp", "compute.cpp", "compute_complex.cpp", "compute_grid_clusters.cpp", "dump.cpp",
    "fixgrid_ave.cpp", "integrate.cpp", "compute_pair.cpp", "fixgrid_gradphi.cpp", "fixatom_drag.cpp",
    "pair_gridatom_lj_ish_linear.cpp", "read_dump.cpp", "conjugate.cpp", "conjugate_volfrac.cpp", "smatrix.cpp",
]
# -ffp-contract=off: no fused multiply-adds, on x86 and Arm alike (the oracle is built the same way)
FLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-w"]


def available():
    return all(os.path.exists(os.path.join(REF_SRC, s)) for s in SOURCES)


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False):
    if not available():
        return None
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "include"), "-I" + REF_SRC]
    shim_hdrs = []
    for root, _, files in os.walk(os.path.join(HERE, "include")):
        shim_hdrs += [os.path.join(root, f) for f in files]
    units = [(os.path.join(REF_SRC, s), os.path.join(OBJ, s.replace(".cpp", ".o"))) for s in SOURCES]
    units += [(os.path.join(HERE, s), os.path.join(OBJ, "refpin_" + s.replace(".cpp", ".o")))
              for s in ("standins.cpp", "driver.cpp")]
    jobs = [["g++"] + FLAGS + inc + ["-c", src, "-o", obj] for src, obj in units
            if force or _newer(obj, [src] + shim_hdrs)]
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for j, r in zip(jobs, ex.map(lambda j: subprocess.run(j, capture_output=True, text=True), jobs)):
                if r.returncode != 0:
                    raise RuntimeError("reference build failed: %s\n%s" % (" ".join(j), r.stderr[-4000:]))
    objs = [o for _, o in units]
    if force or _newer(EXE, objs):
        subprocess.check_call(["g++", "-o", EXE] + objs)
    return EXE


if __name__ == "__main__":
    print(build(force=True))

"""Build recipe of libphafd_gpu.so (sm_103a) and the phafd_gpu host program.

Every CUDA translation unit is compiled by nvcc for sm_103a only, in
parallel, then linked into phafd_gb300/_build/libphafd_gpu.so.  The host
program (a C++ input-script interpreter over the C ABI) links against it.
Outputs stay inside the repository tree (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libphafd_gpu.so")
EXE = os.path.join(OUT, "phafd_gpu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
CU_SOURCES = ["ctx.cu", "bead_kernels.cu", "noalloc.cu", "fno.cu", "clusters.cu",
              "grid_f32_x.cu", "grid_f32_y.cu", "grid_f32_z.cu", "grid_f32_zf.cu",
              "grid_f64_x.cu", "grid_f64_y.cu", "grid_f64_z.cu", "grid_f64_zf.cu"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "phafd_gpu.h"))
    hs.append(os.path.join(ROOT, "include", "phafd_fno.h"))
    return hs


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([nv] + NVFLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(j), r.stdout, r.stderr))
                if verbose and r.stderr:
                    print(r.stderr)
    if force or _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call([nv] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    host_srcs = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST))] if os.path.isdir(HOST) else []
    host_hdrs = [f for f in host_srcs if f.endswith(".hpp")]
    host_srcs = [f for f in host_srcs if f.endswith(".cpp")]
    if host_srcs and (force or _newer(EXE, host_srcs + host_hdrs + [LIB] + hdrs)):
        tmp = EXE + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-o", tmp] + host_srcs +
                              ["-I" + os.path.join(ROOT, "include"), "-L" + OUT, "-lphafd_gpu",
                               "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, EXE)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))

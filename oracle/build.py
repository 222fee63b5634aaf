"""Build recipe for the FP64 CPU oracle (test infrastructure only).

Compiles oracle/phafd_oracle.cpp into oracle/_build/libphafd_oracle.so with
g++.  -ffp-contract=off keeps the arithmetic free of FMA contraction on both
x86-64 and aarch64 hosts, so the oracle computes the same bits on either.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libphafd_oracle.so")
SRC = os.path.join(HERE, "phafd_oracle.cpp")
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "phafd_oracle.h"),
            os.path.join(HERE, "..", "include", "phafd_gpu.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + FLAGS + ["-o", tmp, SRC])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

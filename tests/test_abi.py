"""The C-ABI library builds, loads without a GPU, and exports every symbol
that include/phafd_gpu.h declares."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="phafd_gpu.h"):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(phafd_\w+)\s*\(", txt, flags=re.M)))


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_exports_every_declared_symbol():
    from phafd_gb300 import build as B
    lib = B.build()
    L = ctypes.CDLL(lib)
    syms = declared_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    from phafd_gb300 import gpu
    assert sorted(gpu.EXPORTS) == syms


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_exports_the_learned_propagator():
    from phafd_gb300 import build as B
    L = ctypes.CDLL(B.build())
    syms = declared_symbols("phafd_fno.h")
    assert len(syms) >= 10
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    from phafd_gb300 import fno
    assert sorted(fno.EXPORTS) == syms
    L.phafd_fno_param_count.restype = ctypes.c_size_t
    assert L.phafd_fno_param_count() == fno.param_count()

"""The C-ABI library loads without a GPU and exports every entry point that
include/igapgpu.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "igapgpu.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(igapgpu_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("igapgpu_assm_init", "igapgpu_residual", "igapgpu_tangent", "igapgpu_matmult",
              "igapgpu_solve", "igapgpu_finalize"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import igap4_gb300 as ig
    if not os.path.exists(ig.LIBPATH):
        from igap4_gb300 import build
        build.build()
    lib = ctypes.CDLL(ig.LIBPATH)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_no_gpu_means_error_not_fallback():
    """Without a GPU the context cannot be created: the library reports an
    error instead of computing on the CPU."""
    import numpy as np
    import igap4_gb300 as ig
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    knots, w, X = ig.beam_mesh((2, 2, 2))
    with pytest.raises(ig.IgapGpuError):
        ig.Assembly((2, 2, 2), knots, w, X)

"""The allocation-free 2-norm (igapgpu_norm2_noalloc) against the regular
igapgpu_norm2, through the C ABI.

Callers that cannot allocate device memory -- applications whose pool
allocator owns the GPU's memory, or code that must not trigger the
device-wide synchronisation of cudaMalloc / cudaFree -- use the variant whose
scratch is a fixed array inside the library.  This file is collected last so
that a failure here does not hide any other test; it also passes on its own
in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import igap4_gb300 as ig

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as the other FP64 GPU tests
MAX_N = 8192 * 4096


def _noalloc():
    f = ig.lib().igapgpu_norm2_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_norm2_noalloc_matches_norm2_twice():
    torch = pytest.importorskip("torch")
    knots, w, X = ig.beam_mesh((16, 4, 4), (4.0, 1.0, 1.0))
    A = ig.Assembly((16, 4, 4), knots, w, X, law=ig.LAW_LINGRAD)
    f = _noalloc()
    rng = np.random.default_rng(123)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):  # two calls in a row share the scratch array
        x = torch.tensor(rng.standard_normal(A.ndof) * (call + 1), device="cuda")
        ref = A.norm2(x)
        out_h = ctypes.c_double(-1.0)
        rc = f(ctypes.c_void_p(x.data_ptr()), A.ndof, ctypes.byref(out_h), ctypes.c_void_p(stream))
        assert rc == 0, ig.lib().igapgpu_last_error()
        assert abs(out_h.value - ref) <= TOL * ref
        out_d = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        rc = f(ctypes.c_void_p(x.data_ptr()), A.ndof, ctypes.c_void_p(out_d.data_ptr()),
               ctypes.c_void_p(stream))
        assert rc == 0, ig.lib().igapgpu_last_error()
        torch.cuda.synchronize()
        assert abs(out_d.item() - ref) <= TOL * ref


def test_norm2_noalloc_rejects_oversize_and_host_input():
    torch = pytest.importorskip("torch")
    f = _noalloc()
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = ctypes.c_double()
    rc = f(ctypes.c_void_p(x.data_ptr()), MAX_N + 1, ctypes.byref(out), None)
    assert rc == -1
    assert b"exceeds the maximum" in ig.lib().igapgpu_last_error()
    h = np.ones(4)
    rc = f(ctypes.c_void_p(h.ctypes.data), 4, ctypes.byref(out), None)
    assert rc == -1

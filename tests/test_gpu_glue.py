"""The IGAP4-facing C glue (Residual_gpu / Tangent_gpu / MatMult_gpu with the
reference's callback signatures, reading a Core built like IGAPAssmInit
leaves it) against the oracle.  The PETSc objects are the oracle's
single-rank stand-ins."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_glue():
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "glue_test.so")
    ig.lib()  # the device library must exist
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-Wall", "-Wno-unused-function",
           "-I", os.path.join(ROOT, "oracle", "stub"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "igap4_gb300", "host"),
           os.path.join(ROOT, "igap4_gb300", "host", "igapgpu_igap.c"),
           os.path.join(ROOT, "tests", "c", "glue_driver.c"),
           os.path.join(ROOT, "oracle", "stub", "stub_impl.c"),
           "-L", os.path.join(ROOT, "igap4_gb300"), "-ligapgpu",
           "-Wl,-rpath," + os.path.join(ROOT, "igap4_gb300"), "-ldl", "-o", so]
    subprocess.run(cmd, check=True)
    return ctypes.CDLL(so)


@pytest.mark.parametrize("law,nelem", [(po.LAW_LINGRAD, (6, 3, 2)), (po.LAW_GRADELAST, (3, 3, 3)),
                                       (po.LAW_GRADELASTTIME, (3, 2, 2))])
def test_glue_callbacks_vs_oracle(law, nelem):
    sp = pytest.importorskip("scipy.sparse")
    lib = build_glue()
    bct, neu = po.clamp_bc((0,), 1, (0.0, 1e-3, -1e-3))
    prob = po.Problem(nelem=nelem, law=law, bc_type=bct, neumann=neu)
    knots, w, X = po.mesh_beam(prob)
    U = po.random_state(prob, 41)
    n = prob.ndof
    orc = po.OracleCase(prob)
    RR = np.zeros(n)
    rowptr = np.zeros(n + 1, np.int64)
    cols = np.zeros(orc.nnz, np.int32)
    vals = np.zeros(orc.nnz)
    nnz = ctypes.c_long()
    x = np.random.default_rng(2).standard_normal(n)
    Kx = np.zeros(n)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nel = np.array(nelem, np.int32)
    rc = lib.glue_run(P(nel), P(knots), P(w), P(X), law, P(prob.params()),
                      P(np.ascontiguousarray(bct, np.int32)), P(neu), P(np.ascontiguousarray(U)),
                      P(RR), P(rowptr), P(cols), P(vals), ctypes.byref(nnz), P(x), P(Kx))
    assert rc == 0, ig.lib().igapgpu_last_error()
    R0 = orc.residual(U)
    assert np.linalg.norm(RR - R0) <= 1e-12 * np.linalg.norm(R0)
    assert nnz.value == orc.nnz
    r2, c2 = orc.pattern()
    np.testing.assert_array_equal(rowptr, r2)
    np.testing.assert_array_equal(cols, c2)
    V0 = orc.tangent(U)
    assert np.linalg.norm(vals - V0) <= 1e-12 * np.linalg.norm(V0)
    K = sp.csr_matrix((V0, c2, r2), shape=(n, n))
    assert np.linalg.norm(Kx - K @ x) <= 1e-12 * np.linalg.norm(K @ x)

"""The IGAP4-facing C glue (Residual_gpu / Tangent_gpu with the reference's
SNES callback signatures, MatMult_gpu / MatGetDiagonal_gpu as the operations
of a MATSHELL, reading a Core built like IGAPAssmInit leaves it) against the
oracle, and the reference's solver set-up and Newton loop driving them
through the registered pointers.  The PETSc objects are the oracle's
single-rank stand-ins."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po

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
           "-Wl,-rpath," + os.path.join(ROOT, "igap4_gb300"), "-ldl", "-lm", "-o", so]
    subprocess.run(cmd, check=True)
    return ctypes.CDLL(so)


@pytest.mark.gpu
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


def _snes_run(lib, prob, U0, restart=200):
    knots, w, X = po.mesh_beam(prob)
    U = np.ascontiguousarray(U0, np.float64).copy()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nel = np.array(prob.nelem, np.int32)
    nits, kits, reason = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    fn = ctypes.c_double()
    rc = lib.glue_snes_run(P(nel), P(knots), P(w), P(X), prob.law, P(prob.params()),
                           P(np.ascontiguousarray(prob.bc_type, np.int32)), P(np.ascontiguousarray(prob.neumann)),
                           P(U), restart, ctypes.byref(nits), ctypes.byref(kits), ctypes.byref(reason),
                           ctypes.byref(fn))
    assert rc == 0, ig.lib().igapgpu_last_error()
    return U, nits.value, kits.value, reason.value, fn.value


@pytest.mark.gpu
def test_snes_drives_gpu_callbacks_linear():
    """The reference's Newton set-up (abstol 1e-10, one Newton step per
    SNESSolve inside the outer loop) drives Residual_gpu, Tangent_gpu and the
    MATSHELL multiply through the registered pointers to the direct-solve
    answer of the linear law."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    lib = build_glue()
    bct, neu = po.clamp_bc((0,), 1, (0.0, 1e-3, -1e-3))
    prob = po.Problem(nelem=(6, 3, 2), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    U0 = po.random_state(prob, 5)[0] * 0.1
    U, nits, kits, reason, fn = _snes_run(lib, prob, U0)
    assert reason == 2 and fn <= 1e-10, (reason, fn)
    assert nits >= 1 and kits >= 1
    orc = po.OracleCase(prob)
    r2, c2 = orc.pattern()
    K = sp.csr_matrix((orc.tangent(U0[None]), c2, r2), shape=(prob.ndof, prob.ndof)).tocsc()
    # the tangent has the Dirichlet rows and columns eliminated: the first
    # exact step puts the Dirichlet values in place, the second is then exact
    U1 = U0 - spla.spsolve(K, orc.residual(U0[None]))
    Ustar = U1 - spla.spsolve(K, orc.residual(U1[None]))
    # |F| <= 1e-10 leaves the state within the conditioning of the system
    assert np.linalg.norm(U - Ustar) <= 1e-6 * np.linalg.norm(Ustar)
    assert np.linalg.norm(orc.residual(U[None])) <= 1e-9


@pytest.mark.gpu
def test_snes_drives_gpu_callbacks_gradient_law():
    """Same loop on the reference's static gradient law: the stand-in SNES
    reaches |F| <= 1e-10 through the GPU callbacks, the oracle's residual at
    the result agrees, and the device Newton solver finds the same state."""
    lib = build_glue()
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(3, 2, 2), law=po.LAW_GRADELAST, bc_type=bct, neumann=neu)
    U0 = np.zeros(prob.ndof)
    U, nits, kits, reason, fn = _snes_run(lib, prob, U0)
    assert reason == 2 and fn <= 1e-10, (reason, fn)
    orc = po.OracleCase(prob)
    assert np.linalg.norm(orc.residual(U[None])) <= 1e-9
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=prob.law, par=prob.params(), bc_type=bct, neumann=neu)
    Ud = np.zeros(prob.ndof)
    st = A.solve(Ud, snes_abstol=1e-10, ksp_rtol=1e-8, ksp_max_it=100000)
    assert st["converged"]
    assert np.linalg.norm(U - Ud) <= 1e-6 * max(np.linalg.norm(Ud), 1e-30)


def test_glue_error_codes():
    """Failures come back as positive PETSc error classes (no GPU needed:
    nothing reaches the device)."""
    lib = build_glue()
    codes = np.zeros(6, np.int32)
    assert lib.glue_errors(codes.ctypes.data_as(ctypes.c_void_p)) == 0
    PETSC_ERR_MEM, PETSC_ERR_ARG_WRONGSTATE, PETSC_ERR_LIB = 55, 73, 76
    assert list(codes) == [PETSC_ERR_ARG_WRONGSTATE] * 4 + [PETSC_ERR_LIB, PETSC_ERR_MEM]

"""Batched instances (one persistent launch per kernel over a colour-major
work queue of every instance's elements) against the single-instance path.

The per-element arithmetic and the order in which each CSR slot receives its
element contributions (colour by colour) are the same in both paths, so the
batch must reproduce every instance's residual and tangent bit for bit, in
FP64 and in split precision, under every schedule.  The single-instance path
itself is checked against the reference in test_gpu_assembly.py.
"""
import numpy as np
import pytest

import igap4_gb300 as ig

pytestmark = pytest.mark.gpu

SIZES = [(5, 2, 3), (8, 3, 2), (3, 3, 3), (6, 2, 2), (2, 2, 2), (9, 4, 3)]


def instances(law, seed=0, sizes=SIZES):
    rng = np.random.default_rng(seed)
    bct, neu = ig.clamp_bc((0,), traction_face=1, traction=(0.0, 0.0, -1e-3))
    out = []
    for k, nelem in enumerate(sizes):
        knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0), perturb=(k % 2 == 1))
        if law == ig.LAW_LINGRAD:
            par = [rng.uniform(0.5, 2.0), rng.uniform(0.5, 2.0), rng.uniform(0.02, 0.2), 0, 0, 0, 0, 0, 0]
        else:
            par = list(ig.LAW_DEFAULT_PAR[law])
            par[2] *= rng.uniform(0.8, 1.2)
        out.append(dict(nelem=nelem, knots=knots, w=w, X=X, par=par, bc_type=bct, neumann=neu))
    return out


def singles(insts, law, prec):
    out = []
    for inst in insts:
        A = ig.Assembly(inst["nelem"], inst["knots"], inst["w"], inst["X"], law=law, par=inst["par"],
                        bc_type=inst["bc_type"], neumann=inst["neumann"])
        A.set_precision(prec)
        out.append(A)
    return out


def batch_state(B, seed):
    return np.random.default_rng(seed).uniform(-1e-2, 1e-2, B.ndof)


def compare_to_singles(B, As, U):
    RR = B.residual(U.copy())
    vals = B.tangent(U.copy())
    rowptr, cols = B.pattern()
    for i, A in enumerate(As):
        a, e = B.dof_off[i], B.dof_off[i + 1]
        Ui = np.ascontiguousarray(U[a:e])
        np.testing.assert_array_equal(RR[a:e], A.residual(Ui.copy()))
        rp, cc = A.pattern()
        np.testing.assert_array_equal(rowptr[a:e + 1] - rowptr[a], rp)
        np.testing.assert_array_equal(cols[rowptr[a]:rowptr[e]], cc + a)
        np.testing.assert_array_equal(vals[rowptr[a]:rowptr[e]], A.tangent(Ui.copy()))
    return RR, vals


@pytest.mark.parametrize("law,cached", [(ig.LAW_LINGRAD, "1"), (ig.LAW_LINGRAD, "0"), (ig.LAW_GRADELAST, "1")])
@pytest.mark.parametrize("prec", [ig.PREC_FP64, ig.PREC_SPLIT])
def test_batch_bit_identical_to_single_instances(law, cached, prec, monkeypatch):
    # batches evaluate nonlinear laws inside the element kernels; so do the
    # single instances here (their all-points law launch is compared with this
    # in test_gpu_assembly.py: identical in FP64, within the split bound in split)
    monkeypatch.setenv("IGAPGPU_LAW_PRECOMPUTE", "0")
    # the FP64 residual kernel in split mode for both (the double-FP32
    # residuals are compared with FP64 in test_batch_split_residual_double_fp32
    # and test_gpu_split.py)
    monkeypatch.setenv("IGAPGPU_RES_DF", "0")
    # linear law, split: Gram operands cached (sqrt(w) folded in) or built in the kernel
    monkeypatch.setenv("IGAPGPU_TC_GRAM_CACHE", cached)
    insts = instances(law, seed=3)
    B = ig.BatchAssembly(insts, law=law)
    B.set_precision(prec)
    As = singles(insts, law, prec)
    assert B.ninst == len(insts)
    assert B.ndof == sum(A.ndof for A in As) and B.nnz == sum(A.nnz for A in As)
    assert B.nelem_total == sum(A.nelem_total for A in As)
    compare_to_singles(B, As, batch_state(B, 5))


def test_batch_split_residual_double_fp32(monkeypatch):
    """In split mode the batch evaluates the linear law's residual in
    double-FP32 arithmetic (one launch over every element of every instance,
    then a gather per DOF in a fixed element order): within 1e-13 of the FP64
    element kernel per instance, the same bits on every call, and
    IGAPGPU_RES_DF=0 gives back the FP64 kernel."""
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=21)
    B = ig.BatchAssembly(insts, law=law)
    U = batch_state(B, 22)
    R64 = B.residual(U.copy())
    B.set_precision(ig.PREC_SPLIT)
    Rdf = B.residual(U.copy())
    np.testing.assert_array_equal(B.residual(U.copy()), Rdf)
    assert not np.array_equal(Rdf, R64)  # the pair path ran
    for i in range(B.ninst):
        a, e = B.dof_off[i], B.dof_off[i + 1]
        assert np.linalg.norm(Rdf[a:e] - R64[a:e]) <= 1e-13 * np.linalg.norm(R64[a:e])
    monkeypatch.setenv("IGAPGPU_RES_DF", "0")
    B0 = ig.BatchAssembly(insts, law=law)
    B0.set_precision(ig.PREC_SPLIT)
    np.testing.assert_allclose(B0.residual(U.copy()), R64, rtol=0, atol=1e-15 * np.abs(R64).max())


def test_every_schedule_gives_the_same_bits():
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=4)
    B = ig.BatchAssembly(insts, law=law)
    B.set_precision(ig.PREC_SPLIT)
    U = batch_state(B, 6)
    ref = (B.residual(U.copy()), B.tangent(U.copy()))
    for sched in ({"grab_fp64": 3, "ctas_per_sm_fp64": 2, "grab_tc": 5, "order": 1},
                  {"grab_fp64": 8, "ctas_per_sm_fp64": 1, "grab_tc": 1, "order": 0},
                  {"grab_fp64": 1, "ctas_per_sm_fp64": 1, "grab_tc": 64, "order": 1}):
        B.schedule = sched
        assert B.schedule == sched
        np.testing.assert_array_equal(B.residual(U.copy()), ref[0])
        np.testing.assert_array_equal(B.tangent(U.copy()), ref[1])
    best, t64, ttc = B.autotune(reps=1, frac=0.5)
    assert best == B.schedule and t64 > 0 and ttc > 0
    np.testing.assert_array_equal(B.residual(U.copy()), ref[0])
    np.testing.assert_array_equal(B.tangent(U.copy()), ref[1])
    with pytest.raises(ig.IgapGpuError):
        B.schedule = {"grab_fp64": 0, "ctas_per_sm_fp64": 1, "grab_tc": 1, "order": 0}


def test_batch_dirichlet_and_norms():
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=7)
    B = ig.BatchAssembly(insts, law=law)
    As = singles(insts, law, ig.PREC_FP64)
    rows, g = B.dirichlet()
    exp = np.concatenate([A.dirichlet()[0] + B.dof_off[i] for i, A in enumerate(As)])
    np.testing.assert_array_equal(rows, exp)
    assert np.all(g == 0.0)
    x = np.random.default_rng(8).standard_normal(B.ndof)
    nrm = B.norms(x)
    exp = np.array([np.linalg.norm(x[B.dof_off[i]:B.dof_off[i + 1]]) for i in range(B.ninst)])
    assert np.max(np.abs(nrm - exp) / exp) <= 1e-14


@pytest.mark.parametrize("graphs", [0, 1])
def test_batch_newton_solves_every_instance(graphs):
    """One Newton-GMRES solve of the block-diagonal system: every instance's
    residual is at the tolerance and its solution matches its own solve."""
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=9, sizes=SIZES[:4])
    B = ig.BatchAssembly(insts, law=law)
    opts = dict(snes_abstol=1e-10, ksp_rtol=1e-11, ksp_restart=60, ksp_max_it=60000, snes_max_it=10,
                use_graphs=graphs)
    U = np.zeros(B.ndof)
    st = B.solve(U, **opts)
    assert st["converged"] == 1, st
    F = B.residual(U.copy())
    assert np.all(B.norms(F) <= 1e-10)
    for i, A in enumerate(singles(insts, law, ig.PREC_FP64)):
        Ui = np.zeros(A.ndof)
        si = A.solve(Ui, **opts)
        assert si["converged"] == 1, si
        seg = U[B.dof_off[i]:B.dof_off[i + 1]]
        assert np.linalg.norm(seg - Ui) <= 1e-7 * np.linalg.norm(Ui)


def test_uneven_batch_properties():
    """Sixteen seeded uneven instances (nx in 8..24, ny = nz in 2..6): the
    split-precision tangent of the linear law is symmetric to FP32 rounding
    and its action matches the FP64 tangent within the split bound."""
    sp = pytest.importorskip("scipy.sparse")
    insts = ig.batch_instances(16, seed=11, nx=(8, 24), nyz=(2, 6))
    B = ig.BatchAssembly(insts, law=ig.LAW_LINGRAD)
    U = B.impose_dirichlet(batch_state(B, 12))  # zero on the clamped DOFs
    rowptr, cols = B.pattern()
    K64 = sp.csr_matrix((B.tangent(U.copy()), cols, rowptr), shape=(B.ndof, B.ndof))
    assert abs(K64 - K64.T).max() <= 1e-12 * abs(K64).max()
    B.set_precision(ig.PREC_SPLIT)
    Ks = sp.csr_matrix((B.tangent(U.copy()), cols, rowptr), shape=(B.ndof, B.ndof))
    x = np.random.default_rng(13).standard_normal(B.ndof)
    assert np.linalg.norm(Ks @ x - K64 @ x) <= 1e-5 * np.linalg.norm(K64 @ x)
    # residual of the linear law: R(U) = R(0) + K U
    R0 = B.residual(np.zeros(B.ndof))
    RU = B.residual(U.copy())
    rows, _ = B.dirichlet()
    free = np.ones(B.ndof, bool)
    free[rows] = False
    d = (RU - R0 - K64 @ U)[free]
    assert np.linalg.norm(d) <= 1e-10 * np.linalg.norm((RU - R0)[free])


def test_batch_spmv_matches_single_instances():
    """The single-instance multiply computes its columns from the stencil; the
    batch multiply reads the stored columns.  Same entries, same order: the
    products agree bit for bit."""
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=14)
    B = ig.BatchAssembly(insts, law=law)
    As = singles(insts, law, ig.PREC_FP64)
    U = batch_state(B, 15)
    B.tangent_internal(U.copy())
    x = np.random.default_rng(16).standard_normal(B.ndof)
    y = B.matmult(x)
    for i, A in enumerate(As):
        a, e = B.dof_off[i], B.dof_off[i + 1]
        A.tangent_internal(np.ascontiguousarray(U[a:e]))
        np.testing.assert_array_equal(y[a:e], A.matmult(np.ascontiguousarray(x[a:e])))


def test_bounded_wait_expires_and_context_survives():
    """Failure detection without a fault: a device wait on a counter that
    nothing increments gives up after its poll limit and reports error word 3;
    a wait that is satisfied reports 0; a batch assembles correctly afterwards."""
    assert ig.wait_selftest(1, 1 << 14) == 3
    assert ig.wait_selftest(0, 1 << 14) == 0
    law = ig.LAW_LINGRAD
    insts = instances(law, seed=17, sizes=SIZES[:3])
    B = ig.BatchAssembly(insts, law=law)
    As = singles(insts, law, ig.PREC_FP64)
    compare_to_singles(B, As, batch_state(B, 18))

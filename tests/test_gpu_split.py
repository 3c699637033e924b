"""Tensor-core (tcgen05, TF32x3) split-precision tangent.

* the tcgen05 self-test GEMM reproduces an exact integer product;
* the split tangent agrees with the FP64 tangent within the stated bound
  (relative 2-norm error <= 1e-5, measured ~4e-6; TF32 hi+lo operands keep ~21 bits, the
  FP32 tensor-memory accumulation dominates), for all three laws and every GEMM form
  of the linear law (Gram form from cached sqrt(w)-weighted operands, Gram form built
  from the FP32 geometry cache, and the two-stage form used by the other laws);
* the residual of the tensor-core modes runs in double-FP32 arithmetic (pairs of
  floats, compensated dot products): the linear law's whole element loop, and for
  the reference's laws the interpolation of the law's inputs and the projection
  around the FP64 law; within 1e-12 of the FP64 residual (measured ~1e-15) and of
  the CPU oracle.
"""
import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po

pytestmark = pytest.mark.gpu

SPLIT_TOL = 1e-5
DF_TOL = 1e-12  # double-FP32 residual of the linear law vs FP64


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_tcgen05_selftest_exact():
    D, E = ig.tc_selftest(0)
    assert np.array_equal(D, E), f"max |D-E| = {np.abs(D - E).max()}"


@pytest.mark.parametrize("law,nelem,perturb,form", [
    (po.LAW_LINGRAD, (8, 4, 3), False, "cached"),  # Gram-form GEMM on cached operands (tc_gram.cu)
    (po.LAW_LINGRAD, (5, 3, 4), True, "cached"),
    (po.LAW_LINGRAD, (5, 3, 4), True, "gram"),     # Gram-form GEMM built from the FP32 geometry cache
    (po.LAW_LINGRAD, (8, 4, 3), False, "dense"),   # two-stage GEMM (tc_tangent.cu)
    (po.LAW_GRADELAST, (4, 4, 4), True, "dense"),
    (po.LAW_GRADELASTTIME, (3, 3, 4), False, "dense"),
])
def test_split_tangent_vs_fp64(law, nelem, perturb, form, monkeypatch):
    if form == "dense" and law == po.LAW_LINGRAD:
        monkeypatch.setenv("IGAPGPU_TC_DENSE", "1")
    if form == "gram":
        monkeypatch.setenv("IGAPGPU_TC_GRAM_CACHE", "0")
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=nelem, law=law, perturb=perturb, bc_type=bct, neumann=neu)
    U = po.random_state(prob, 77)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L, prob.p, prob.perturb)
    A = ig.Assembly(prob.nelem, knots, w, X, law=law, par=prob.params(), bc_type=bct, neumann=neu)
    A.set_state(U)
    K64 = A.tangent()
    R64 = A.residual()
    n0 = ig.launch_count()
    A.set_precision(ig.PREC_SPLIT)
    # the cached form builds its operands once, in one launch, when split
    # precision is set; the linear law's residual pairs in one more
    lin = law == po.LAW_LINGRAD
    assert ig.launch_count() - n0 == (1 if lin and form != "gram" else 0) + (1 if lin else 0)
    Ks = A.tangent()
    Rs = A.residual()
    e = rel(Ks, K64)
    print(f"split tangent rel err {e:.3e}")
    assert e <= SPLIT_TOL
    er = rel(Rs, R64)
    print(f"double-FP32 residual rel err {er:.3e}")
    assert er <= DF_TOL
    assert not np.array_equal(Rs, R64)  # the pair path ran
    np.testing.assert_array_equal(A.residual(), Rs)  # deterministic
    # fused assemble in split mode = the residual above + split tangent
    RR = np.zeros(A.ndof)
    V = np.zeros(A.nnz)
    A.assemble(None, RR, V)
    np.testing.assert_array_equal(RR, Rs)
    assert rel(V, K64) <= SPLIT_TOL


@pytest.mark.parametrize("cached", ["1", "0"])
@pytest.mark.parametrize("nquad", [3, 4])
def test_split_gram_partial_chunks(nquad, cached, monkeypatch):
    """Gram-form split tangent with 27 points per element (chunks of 8, 8, 8, 3)
    and with 64, against the FP64 tangent of the same quadrature, from cached
    operands and built in the kernel."""
    monkeypatch.setenv("IGAPGPU_TC_GRAM_CACHE", cached)
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh((6, 3, 2), (4.0, 1.0, 1.0), 2, True)
    A = ig.Assembly((6, 3, 2), knots, w, X, law=ig.LAW_LINGRAD, par=(1.3, 0.8, 0.12), bc_type=bct,
                    neumann=neu, nquad=nquad)
    U = np.random.default_rng(5).uniform(-1e-2, 1e-2, A.ndof)
    K64 = A.tangent(U.copy())
    A.set_precision(ig.PREC_SPLIT)
    Ks = A.tangent(U.copy())
    assert rel(Ks, K64) <= SPLIT_TOL


def test_split_newton_converges_to_fp64_tolerance():
    """Inexact (split) Jacobian, exact FP64 residual: Newton still reaches the
    FP64 residual tolerance."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(16, 4, 4), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=prob.law, par=prob.params(), bc_type=bct, neumann=neu)
    A.set_precision(ig.PREC_SPLIT)
    U = np.zeros(A.ndof)
    st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-10, ksp_restart=300, ksp_max_it=50000, snes_max_it=20)
    assert st["converged"] == 1, st
    orc = po.OracleCase(prob)
    assert np.linalg.norm(orc.residual(U[None, :])) <= 1e-9


def test_warp_specialised_tangent_bit_identical(monkeypatch):
    """The warp-specialised cached-operand kernel (copies, TF32 split, MMAs and
    scatter on separate warps) performs the same arithmetic in the same order
    as the single-role kernel: the tangents agree bit for bit."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh((9, 4, 5), (4.0, 1.0, 1.0), 2, True)
    A = ig.Assembly((9, 4, 5), knots, w, X, law=ig.LAW_LINGRAD, par=(1.1, 0.9, 0.08), bc_type=bct, neumann=neu)
    A.set_precision(ig.PREC_SPLIT)
    U = np.random.default_rng(8).uniform(-1e-2, 1e-2, A.ndof)
    monkeypatch.setenv("IGAPGPU_TCS_WS", "0")
    K1 = A.tangent(U.copy())
    monkeypatch.setenv("IGAPGPU_TCS_WS", "1")
    K2 = A.tangent(U.copy())
    np.testing.assert_array_equal(K1, K2)


def slab_rows(prob, ix):
    """CSR rows of the control points of x-layer ix (every DOF), and the
    element range whose contributions complete them: the slabs ix-2..ix."""
    nb = prob.nbasis
    per_layer = 3 * nb[1] * nb[2]
    rows = np.arange(ix * per_layer, (ix + 1) * per_layer)
    per_slab = prob.nelem[1] * prob.nelem[2]
    return rows, (ix - 2) * per_slab, (ix + 1) * per_slab


def rows_of(vals, rowptr, rows):
    return np.concatenate([vals[rowptr[r]:rowptr[r + 1]] for r in rows])


@pytest.mark.parametrize("law,nelem", [(po.LAW_LINGRAD, (32, 8, 8)), (po.LAW_LINGRAD, (16, 4, 4)),
                                       (po.LAW_GRADELAST, (16, 4, 4)), (po.LAW_GRADELASTTIME, (16, 4, 4))])
def test_split_and_fp64_vs_cpu_oracle(law, nelem):
    """Both precisions against the FP64 CPU oracle directly, at the sizes of the
    assembly sweep and of the static workload: the full residual, and the
    tangent on the rows of one control-point layer in the middle of the beam
    (the oracle assembles the three element slabs that complete them).  FP64:
    1e-12 relative; split: the stated 1e-5 bound."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=nelem, L=(4.0, 1.0, 1.0), law=law, bc_type=bct, neumann=neu)
    U = po.random_state(prob, 31)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=law, par=prob.params(), bc_type=bct, neumann=neu)
    A.set_state(U)
    R64, K64 = A.residual(), A.tangent()
    A.set_precision(ig.PREC_SPLIT)
    Ks, Rs = A.tangent(), A.residual()
    orc = po.OracleCase(prob)
    rowptr, _ = orc.pattern()
    Ro = orc.residual(U)
    assert rel(R64, Ro) <= 1e-12
    ers = rel(Rs, Ro)
    print(f"law {law} {nelem}: split-mode residual {ers:.2e} vs the CPU oracle")
    assert ers <= (DF_TOL if law == po.LAW_LINGRAD else 1e-12)
    ix = nelem[0] // 2 + 1
    rows, e0, e1 = slab_rows(prob, ix)
    Ko = rows_of(orc.tangent_elements(U, e0, e1), rowptr, rows)
    e64, es = rel(rows_of(K64, rowptr, rows), Ko), rel(rows_of(Ks, rowptr, rows), Ko)
    print(f"law {law} {nelem}: FP64 {e64:.2e}, split {es:.2e} vs the CPU oracle")
    assert e64 <= 1e-12
    assert es <= SPLIT_TOL


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME])
@pytest.mark.parametrize("nquad", [4, 3])
def test_law_df_residual(law, nquad, monkeypatch):
    """The reference's laws in the tensor-core modes: the law's inputs by pair
    interpolation (the history differences formed on the nodal values in
    FP64), the FP64 law at every point, the projection on pairs.  Within
    1e-12 of the FP64 residual and of the CPU oracle for random history
    levels and for nearby levels sampled from a motion at the default time
    step (the inertia term's second difference); the same bits on every call and in the fused
    assembly; IGAPGPU_RES_DF=0 gives back the FP64 residual bit for bit."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(5, 3, 4), law=law, perturb=True, bc_type=bct, neumann=neu, nquad=nquad)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L, prob.p, prob.perturb)
    mk = lambda: ig.Assembly(prob.nelem, knots, w, X, law=law, par=prob.params(), bc_type=bct, neumann=neu,
                             nquad=nquad)
    rng = np.random.default_rng(41)
    states = [po.random_state(prob, 42)]
    if prob.torder >= 2:  # u_{n-1}, u_n, u sampled from a smooth motion
        dt = prob.params()[7]
        base = rng.uniform(-1e-2, 1e-2, prob.ndof)
        # |u| / (|a| dt^2) ~ 40: the FP64 residual of the comparison keeps ~1e-14
        v, a = rng.uniform(-1.0, 1.0, prob.ndof), rng.uniform(-1e3, 1e3, prob.ndof)
        states.append(np.stack([base + 2 * v * dt + a * dt * dt, base + v * dt, base]))
    A = mk()
    R64, K64 = [], []
    for U in states:
        A.set_state(U)
        R64.append(A.residual())
        K64.append(A.tangent())
    orc = po.OracleCase(prob)
    for prec in (ig.PREC_SPLIT, ig.PREC_OZAKI):
        A.set_precision(prec)
        for U, R, K in zip(states, R64, K64):
            A.set_state(U)
            if prec == ig.PREC_SPLIT:  # the FP32 law's tangent, chunks loaded entry-major
                assert rel(A.tangent(), K) <= SPLIT_TOL
            Rd = A.residual()
            er, eo = rel(Rd, R), rel(Rd, orc.residual(U))
            print(f"law {law} nquad {nquad} prec {prec}: double-FP32 residual {er:.2e} vs FP64, {eo:.2e} vs oracle")
            assert er <= DF_TOL and eo <= DF_TOL
            assert not np.array_equal(Rd, R)  # the pair path ran
            np.testing.assert_array_equal(A.residual(), Rd)
            if prec == ig.PREC_SPLIT:
                RR, V = np.zeros(A.ndof), np.zeros(A.nnz)
                A.assemble(None, RR, V)
                np.testing.assert_array_equal(RR, Rd)
    monkeypatch.setenv("IGAPGPU_RES_DF", "0")
    B = mk()
    B.set_precision(ig.PREC_SPLIT)
    for U, R in zip(states, R64):
        B.set_state(U)
        np.testing.assert_array_equal(B.residual(), R)


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME])
@pytest.mark.parametrize("nquad", [4, 3])
def test_prefetching_tangent_bit_identical(law, nquad, monkeypatch):
    """The reference laws' split tangent with the law outputs precomputed: the
    form that loads the next chunk's basis and law outputs into registers
    during the current chunk performs the same arithmetic as the point_setup
    form (IGAPGPU_TC_PREFETCH=0): the same bits."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(5, 3, 4), law=law, perturb=True, bc_type=bct, neumann=neu, nquad=nquad)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L, prob.p, prob.perturb)
    A = ig.Assembly(prob.nelem, knots, w, X, law=law, par=prob.params(), bc_type=bct, neumann=neu, nquad=nquad)
    A.set_state(po.random_state(prob, 51))
    A.set_precision(ig.PREC_SPLIT)
    K1 = A.tangent()
    monkeypatch.setenv("IGAPGPU_TC_PREFETCH", "0")
    K0 = A.tangent()
    np.testing.assert_array_equal(K1, K0)


# ---------------------------------------------------------- FP64-quality mode
OZAKI_TOL = 1e-9


def test_tcgen05_selftest_bf16_exact():
    """The BF16 (kind::f16) MMA path of the FP64-quality tangent reproduces an
    exact integer product."""
    D, E = ig.tc_selftest(2)
    assert np.array_equal(D, E), f"max |D-E| = {np.abs(D - E).max()}"


@pytest.mark.parametrize("nelem,perturb,nquad", [((8, 4, 3), False, 4), ((5, 3, 4), True, 4),
                                                 ((6, 3, 2), True, 3)])
def test_ozaki_tangent_vs_fp64(nelem, perturb, nquad):
    """Tangent from error-free BF16 slices of the Gram operands (one
    power-of-two scale per row, exact leading product): within 1e-9 of the
    FP64 tangent; the residual (double-FP32) within 1e-12 of the FP64 one."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0), 2, perturb)
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_LINGRAD, par=(1.3, 0.8, 0.12), bc_type=bct, neumann=neu,
                    nquad=nquad)
    U = np.random.default_rng(3).uniform(-1e-2, 1e-2, A.ndof)
    K64, R64 = A.tangent(U.copy()), A.residual(U.copy())
    n0 = ig.launch_count()
    A.set_precision(ig.PREC_OZAKI)
    assert ig.launch_count() - n0 == 2  # slices and residual pairs are built once, one launch each
    Ko, Ro = A.tangent(U.copy()), A.residual(U.copy())
    e = rel(Ko, K64)
    er = rel(Ro, R64)
    print(f"FP64-quality tensor-core tangent rel err {e:.3e}, residual {er:.3e}")
    assert e <= OZAKI_TOL
    assert er <= DF_TOL
    RR, V = np.zeros(A.ndof), np.zeros(A.nnz)
    A.assemble(U.copy(), RR, V)
    np.testing.assert_array_equal(RR, Ro)
    assert rel(V, K64) <= OZAKI_TOL
    # twice in a row: the same values (the slices are state independent)
    np.testing.assert_array_equal(A.tangent(U.copy()), Ko)


@pytest.mark.parametrize("nquad", [4, 3])
def test_df_residual_switch_and_large_state(nquad, monkeypatch):
    """IGAPGPU_RES_DF=0 keeps the FP64 residual kernel in the tensor-core
    modes (bit-identical to FP64 mode); with it on, the double-FP32 residual
    stays within 1e-12 of FP64 for a state with a large rigid translation (the
    interpolation's terms cancel) and for a state near 1e3."""
    nelem = (6, 3, 3)
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0), 2, True)
    rng = np.random.default_rng(11)
    mk = lambda: ig.Assembly(nelem, knots, w, X, law=ig.LAW_LINGRAD, par=(1.3, 0.8, 0.12), bc_type=bct,
                             neumann=neu, nquad=nquad)
    A = mk()
    n = A.ndof
    states = [rng.uniform(-1e-2, 1e-2, n), 5.0 + rng.uniform(-1e-3, 1e-3, n), rng.uniform(-1e3, 1e3, n)]
    R64 = [A.residual(U.copy()) for U in states]
    monkeypatch.setenv("IGAPGPU_RES_DF", "0")
    B = mk()
    B.set_precision(ig.PREC_SPLIT)
    for U, R in zip(states, R64):
        np.testing.assert_array_equal(B.residual(U.copy()), R)
    monkeypatch.delenv("IGAPGPU_RES_DF")
    A.set_precision(ig.PREC_OZAKI)
    for U, R in zip(states, R64):
        er = rel(A.residual(U.copy()), R)
        print(f"nquad {nquad}: double-FP32 residual rel err {er:.3e}")
        assert er <= DF_TOL


def test_ozaki_vs_cpu_oracle_sweep_mesh():
    """At the 32x8x8 size of the assembly sweep, against the FP64 CPU oracle on
    the rows of one control-point layer."""
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(32, 8, 8), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    U = po.random_state(prob, 31)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=prob.law, par=prob.params(), bc_type=bct, neumann=neu)
    A.set_state(U)
    A.set_precision(ig.PREC_OZAKI)
    Ko = A.tangent()
    orc = po.OracleCase(prob)
    rowptr, _ = orc.pattern()
    rows, e0, e1 = slab_rows(prob, 17)
    err = rel(rows_of(Ko, rowptr, rows), rows_of(orc.tangent_elements(U, e0, e1), rowptr, rows))
    print(f"FP64-quality tensor-core tangent vs CPU oracle: {err:.3e}")
    assert err <= OZAKI_TOL


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME])
def test_ozaki_mode_other_laws_is_fp64(law):
    """The reference's laws have no sliced operands: the FP64-quality mode
    assembles their tangent with the FP64 kernel (the same values)."""
    prob = po.Problem(nelem=(4, 3, 3), law=law)
    U = po.random_state(prob, 6)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=law, par=prob.params())
    A.set_state(U)
    K64 = A.tangent()
    A.set_precision(ig.PREC_OZAKI)
    np.testing.assert_array_equal(A.tangent(), K64)


@pytest.mark.parametrize("prec", [ig.PREC_SPLIT, ig.PREC_OZAKI])
def test_df_matmult_vs_fp64(prec, monkeypatch):
    """The split and FP64-quality modes multiply in double-FP32 arithmetic
    (values and x split into float pairs on the integer pipe, compensated
    row sums).  The same assembled FP64 matrix, multiplied in both modes:
    within 1e-13, for x with exact zeros and for x spanning 1e-30 .. 1e6
    (the out-of-range entries take the FP64 split).  Opt-in
    (IGAPGPU_SPMV_DF=1); without it the FP64 multiply, bit for bit."""
    nelem = (9, 3, 4)
    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0), 2, True)
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_LINGRAD, par=(1.3, 0.8, 0.12), bc_type=bct, neumann=neu)
    rng = np.random.default_rng(17)
    A.tangent(rng.uniform(-1e-2, 1e-2, A.ndof))  # the FP64 matrix, kept by the context
    xs = [rng.standard_normal(A.ndof), rng.standard_normal(A.ndof) * 10.0 ** rng.uniform(-30, 6, A.ndof)]
    xs[0][::7] = 0.0
    y64 = [A.matmult(x.copy()) for x in xs]
    A.set_precision(prec)  # the matrix stays; the multiply changes
    monkeypatch.setenv("IGAPGPU_SPMV_DF", "1")
    for x, y in zip(xs, y64):
        yd = A.matmult(x.copy())
        e = np.linalg.norm(yd - y) / np.linalg.norm(y)
        print(f"double-FP32 multiply rel diff {e:.2e}")
        assert e <= 1e-13
    monkeypatch.delenv("IGAPGPU_SPMV_DF")
    for x, y in zip(xs, y64):
        np.testing.assert_array_equal(A.matmult(x.copy()), y)

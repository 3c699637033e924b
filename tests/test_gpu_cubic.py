"""Cubic C1 elements (degree 3: 64 basis functions, 192 DOFs per element) on
the device in FP64, against the project's C restatement of the reference's
assembly loop with its Cox-de Boor basis (the reference itself takes p = 2
only: eval_Bspline exits for p != 2, src/meshcore_iga.c:293; the restatement
is pinned to the reference at p = 2 in test_oracle.py): residual and tangent
to 1e-12 relative, the degree-3 pattern bit for bit, Newton to the direct
solve; the quadratic-only paths refuse the degree."""
import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def cubic_case(prob):
    knots, w, X = po.mesh_beam(prob)
    kl, o = [], 0
    for n in prob.nelem:
        k = n + 1 + 2 * prob.p
        kl.append(knots[o:o + k])
        o += k
    return ig.Assembly(prob.nelem, kl, w, X, law=prob.law, par=prob.params(), bc_type=prob.bc_type,
                       neumann=prob.neumann, par_dirichlet=prob.par_dirichlet, nquad=prob.nquad, porder=prob.p)


@pytest.mark.parametrize("law,nelem,perturb", [(po.LAW_LINGRAD, (5, 3, 3), True),
                                               (po.LAW_GRADELAST, (4, 3, 3), True),
                                               (po.LAW_GRADELASTTIME, (4, 3, 3), False)])
def test_cubic_assembly_vs_oracle(law, nelem, perturb):
    bct, neu = po.clamp_bc((0,), 1, (0.0, 1e-3, -1e-3))
    neu[6 * 1 + 3 + 2] = 2e-4       # a normal-derivative traction too
    bct[6 * 2:6 * 2 + 6] = 0        # and a second clamped face with affine data
    pdir = np.array([0.0, 1e-3, 0.0, 0.0, 0.0, -2e-3, 0.0, 0.0, 0.0])
    prob = po.Problem(nelem=nelem, L=(2.0, 1.0, 1.0), p=3, perturb=perturb, law=law, bc_type=bct, neumann=neu,
                      par_dirichlet=pdir)
    U = po.random_state(prob, 17)
    A = cubic_case(prob)
    orc = po.OracleCase(prob)
    r1, c1 = A.pattern()
    r2, c2 = orc.pattern()
    np.testing.assert_array_equal(r1, r2)
    np.testing.assert_array_equal(c1, c2)
    A.set_state(U)
    R, K = A.residual(), A.tangent()
    eR, eK = rel(R, orc.residual(U)), rel(K, orc.tangent(U))
    print(f"cubic law {law}: residual {eR:.2e}, tangent {eK:.2e}")
    assert eR <= 1e-12 and eK <= 1e-12


def test_cubic_newton_linear_beam():
    """Clamped cubic beam under a tip traction, linear law: Newton-GMRES on the
    device reaches the direct-solve answer."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(8, 3, 3), L=(4.0, 1.0, 1.0), p=3, law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    A = cubic_case(prob)
    U = np.zeros(A.ndof)
    st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-10, ksp_restart=200, ksp_max_it=50000, orth=1)
    assert st["converged"] == 1, st
    orc = po.OracleCase(prob)
    rowptr, cols = orc.pattern()
    Z = np.zeros((1, A.ndof))
    K = sp.csr_matrix((orc.tangent(Z), cols, rowptr), shape=(A.ndof, A.ndof))
    Ud = -spl.spsolve(K.tocsc(), orc.residual(Z))
    assert rel(U, Ud) <= 1e-7
    assert np.linalg.norm(orc.residual(U[None, :])) <= 1e-9


def test_cubic_refuses_quadratic_only_paths():
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(4, 3, 3), p=3, law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    A = cubic_case(prob)
    for mode in (ig.PREC_SPLIT, ig.PREC_OZAKI):
        with pytest.raises(ig.IgapGpuError):
            A.set_precision(mode)
    with pytest.raises(ig.IgapGpuError):
        A.density()
    A.tangent_internal(np.zeros(A.ndof))
    with pytest.raises(ig.IgapGpuError):
        A.solve(np.zeros(A.ndof), pc=3)

"""Transient three-level scheme driven on the device against a CPU Newton
loop built on the oracle (same law, same seeded load history): converged
trajectories agree to the Newton tolerance."""
import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po
from igap4_gb300.transient import TipLoad, run_transient

pytestmark = pytest.mark.gpu


def cpu_trajectory(prob, load, nsteps, dt, tol=1e-12):
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    hist = np.zeros((3, prob.ndof))  # level 0 iterate, 1 u_n, 2 u_{n-1}
    out = [np.zeros(prob.ndof)]
    for n in range(nsteps):
        t = (n + 1) * dt
        prob.neumann = load.table(t)
        case = po.OracleCase(prob)
        rowptr, cols = case.pattern()
        hist[0] = hist[1]
        for it in range(30):
            R = case.residual(hist)
            if np.linalg.norm(R) < tol:
                break
            K = sp.csr_matrix((case.tangent(hist), cols, rowptr), shape=(prob.ndof, prob.ndof))
            hist[0] -= spl.spsolve(K.tocsc(), R)
        hist[2] = hist[1]
        hist[1] = hist[0]
        out.append(hist[0].copy())
    return np.array(out)


def test_transient_matches_cpu_newton():
    torch = pytest.importorskip("torch")
    dt = 1e-2
    par = np.array(ig.LAW_DEFAULT_PAR[ig.LAW_GRADELASTTIME], dtype=float)
    par[5], par[7] = 1.0, dt
    bct, _ = po.clamp_bc((0,))
    load = TipLoad(seed=3, amax=5e-3)
    prob = po.Problem(nelem=(4, 2, 2), L=(4.0, 1.0, 1.0), law=po.LAW_GRADELASTTIME, par=par,
                      bc_type=bct)
    nsteps = 4
    ref = cpu_trajectory(prob, load, nsteps, dt)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    A = ig.Assembly(prob.nelem, knots, w, X, law=ig.LAW_GRADELASTTIME, par=par, bc_type=bct)
    states, recs = run_transient(A, load, nsteps, dt,
                                 opts=dict(snes_abstol=1e-12, ksp_rtol=1e-12, ksp_restart=300,
                                           ksp_max_it=20000))
    assert all(r.converged == 1 for r in recs), recs
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(states - ref).max() <= 1e-8 * scale


def test_history_shift_and_set_neumann():
    torch = pytest.importorskip("torch")
    prob = po.Problem(nelem=(3, 2, 2), law=po.LAW_GRADELASTTIME)
    knots, w, X = ig.beam_mesh(prob.nelem)
    A = ig.Assembly(prob.nelem, knots, w, X, law=ig.LAW_GRADELASTTIME)
    U = po.random_state(prob, 5)
    A.set_state(U)
    A.shift_history()
    np.testing.assert_array_equal(A.get_history(2), U[1])
    np.testing.assert_array_equal(A.get_history(1), U[0])
    # a traction table change moves the residual by exactly the Neumann load
    R0 = A.residual()
    tab = np.zeros(36)
    tab[6 * 1 + 2] = -1e-3
    A.set_neumann(tab)
    R1 = A.residual()
    bct = np.ones(36, np.int32)
    prob2 = po.Problem(nelem=(3, 2, 2), law=po.LAW_GRADELASTTIME, neumann=tab, bc_type=bct)
    orc = po.OracleCase(prob2)
    Uh = np.stack([A.get_history(0), A.get_history(1), A.get_history(2)])
    np.testing.assert_allclose(R1, orc.residual(Uh), rtol=0, atol=1e-12 * np.abs(R1).max())
    assert np.abs(R1 - R0).max() > 0

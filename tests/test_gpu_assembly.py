"""GPU parity: the CUDA assembly through the C ABI against the reference.

* golden fixtures made by the reference's own code (tests/golden/) -- FP64
  mode must agree to 1e-12 relative (norm-wise), sparsity pattern bit-exact;
* the project's C restatement (oracle/) on larger and edge-case problems;
* size-independent properties at the benchmark size (linearity, symmetry,
  rigid-translation invariance).
"""
import os

import numpy as np
import pytest

import igap4_gb300 as ig
import pyoracle as po
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 mode, relative in the 2-norm


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def gpu_case(prob: po.Problem):
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L, prob.p, prob.perturb)
    return ig.Assembly(prob.nelem, knots, w, X, law=prob.law, par=prob.params(),
                       bc_type=prob.bc_type, neumann=prob.neumann,
                       par_dirichlet=prob.par_dirichlet, nquad=prob.nquad)


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def problem_from_golden(g):
    return po.Problem(nelem=tuple(int(x) for x in g["nelem"]), L=tuple(g["L"]), law=int(g["law"]),
                      perturb=bool(g["perturb"]), par=g["par"], bc_type=g["bc_type"].astype(np.int32),
                      neumann=g["neumann"])


@pytest.mark.parametrize("name", ["g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2"])
def test_golden_full(name):
    g = load(name)
    prob = problem_from_golden(g)
    A = gpu_case(prob)
    A.set_state(g["U"])
    RR = A.residual(np.ascontiguousarray(g["U"][0]))
    assert rel(RR, g["RR"]) <= TOL
    rowptr, cols = A.pattern()
    np.testing.assert_array_equal(rowptr, g["rowptr"])
    np.testing.assert_array_equal(cols, g["cols"])
    vals = A.tangent(np.ascontiguousarray(g["U"][0]))
    assert rel(vals, g["vals"]) <= TOL


@pytest.mark.parametrize("name", ["g_static_beamtest_4x4x4", "g_lingrad_8x2x2"])
def test_golden_summary(name):
    g = load(name)
    prob = problem_from_golden(g)
    A = gpu_case(prob)
    A.set_state(g["U"])
    RR = A.residual()
    assert rel(RR, g["RR"]) <= TOL
    rowptr, cols = A.pattern()
    np.testing.assert_array_equal(rowptr, g["rowptr"])
    assert cols.astype(np.int64).sum() == g["cols_sum"]
    vals = A.tangent()
    assert abs(np.linalg.norm(vals) - g["vals_norm"]) <= TOL * g["vals_norm"]
    np.testing.assert_allclose(vals[g["sample_idx"]], g["sample_vals"], rtol=0,
                               atol=TOL * np.abs(g["sample_vals"]).max())


CASES = [
    # (law, nelem, perturb, L)
    (po.LAW_LINGRAD, (8, 4, 3), False, (4.0, 1.0, 1.0)),
    (po.LAW_GRADELAST, (4, 4, 4), True, (1.0, 1.0, 1.0)),
    (po.LAW_GRADELAST, (5, 3, 4), False, (2.0, 1.0, 1.5)),
    (po.LAW_GRADELASTTIME, (3, 3, 3), False, (1.0, 1.0, 1.0)),
    (po.LAW_GRADELASTTIME, (4, 2, 3), True, (1.0, 1.0, 1.0)),
]


@pytest.mark.parametrize("law,nelem,perturb,L", CASES)
def test_vs_oracle(law, nelem, perturb, L):
    bct, neu = po.clamp_bc((0, 3), 5, (1e-3, 2e-3, -1e-3))
    bct[6 * 1 + 3:6 * 1 + 6] = 1
    neu[6 * 1 + 4] = 5e-4
    prob = po.Problem(nelem=nelem, L=L, law=law, perturb=perturb, bc_type=bct, neumann=neu,
                      par_dirichlet=np.linspace(0.01, 0.09, 9))
    U = po.random_state(prob, 31)
    orc = po.OracleCase(prob)
    A = gpu_case(prob)
    A.set_state(U)
    assert rel(A.residual(), orc.residual(U)) <= TOL
    assert rel(A.tangent(), orc.tangent(U)) <= TOL
    # fused pass gives the same numbers
    RR = np.zeros(A.ndof)
    vals = np.zeros(A.nnz)
    A.assemble(None, RR, vals)
    assert rel(RR, orc.residual(U)) <= TOL
    assert rel(vals, orc.tangent(U)) <= TOL


def test_nquad3_mode_vs_oracle():
    """27-point Gauss mode (nquad = 3): pinned by the oracle only."""
    prob = po.Problem(nelem=(4, 3, 2), law=po.LAW_GRADELAST, nquad=3)
    U = po.random_state(prob, 4)
    orc = po.OracleCase(prob)
    A = gpu_case(prob)
    A.set_state(U)
    assert rel(A.residual(), orc.residual(U)) <= TOL
    assert rel(A.tangent(), orc.tangent(U)) <= TOL


def test_device_pointers_and_history_side_effect():
    torch = pytest.importorskip("torch")
    prob = po.Problem(nelem=(3, 2, 2), law=po.LAW_GRADELAST)
    U = po.random_state(prob, 8)
    A = gpu_case(prob)
    dU = torch.tensor(U[0], device="cuda")
    dR = torch.zeros(A.ndof, dtype=torch.float64, device="cuda")
    dV = torch.zeros(A.nnz, dtype=torch.float64, device="cuda")
    A.residual(dU, dR)
    A.tangent(dU, dV)
    A.synchronize()
    orc = po.OracleCase(prob)
    assert rel(dR.cpu().numpy(), orc.residual(U)) <= TOL
    assert rel(dV.cpu().numpy(), orc.tangent(U)) <= TOL
    # Residual_iga copies U into U_hist[0] (src/assmcore_iga.c:68)
    np.testing.assert_array_equal(A.get_history(0), U[0])


def test_symmetry_and_rigid_translation_full_size():
    """Benchmark-size beam (128 x 32 x 32, linear law): the assembled tangent
    is symmetric, the volume residual of a rigid translation vanishes, and the
    linear law's residual is linear: R(U) - R(0) = K U on free rows."""
    torch = pytest.importorskip("torch")
    nelem = (128, 32, 32)
    knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0))
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_LINGRAD)  # all faces traction-free
    rng = np.random.default_rng(2)
    U = torch.tensor(rng.uniform(-1e-2, 1e-2, A.ndof), device="cuda")
    R = torch.zeros(A.ndof, dtype=torch.float64, device="cuda")
    A.tangent_internal(U)
    A.residual(U, R)
    KU = torch.zeros_like(R)
    A.matmult(U, KU)
    A.synchronize()
    assert (torch.linalg.norm(R - KU) / torch.linalg.norm(R)).item() <= 1e-12
    T = torch.tensor(np.tile([0.3, -0.2, 0.1], A.ndof // 3), device="cuda")
    A.residual(T, R)
    A.synchronize()
    assert torch.abs(R).max().item() <= 1e-12 * torch.abs(KU).max().item() * 10
    # symmetry: x^T K y == y^T K x
    x = torch.tensor(rng.standard_normal(A.ndof), device="cuda")
    y = torch.tensor(rng.standard_normal(A.ndof), device="cuda")
    Kx = torch.zeros_like(x)
    Ky = torch.zeros_like(x)
    A.matmult(x, Kx)
    A.matmult(y, Ky)
    A.synchronize()
    a, b = torch.dot(y, Kx).item(), torch.dot(x, Ky).item()
    assert abs(a - b) <= 1e-12 * abs(a)


def test_spmv_and_diagonal_vs_scipy():
    sp = pytest.importorskip("scipy.sparse")
    prob = po.Problem(nelem=(6, 3, 3), law=po.LAW_GRADELAST)
    U = po.random_state(prob, 5)
    A = gpu_case(prob)
    A.set_state(U)
    A.tangent_internal()
    rowptr, cols = A.pattern()
    vals = A.tangent()
    K = sp.csr_matrix((vals, cols, rowptr), shape=(A.ndof, A.ndof))
    x = np.random.default_rng(1).standard_normal(A.ndof)
    assert rel(A.matmult(x), K @ x) <= 1e-14
    np.testing.assert_array_equal(A.diagonal(), K.diagonal())


def test_gmres_jacobi_solves():
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(8, 2, 2), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    A = gpu_case(prob)
    A.tangent_internal(np.zeros(A.ndof))
    rowptr, cols = A.pattern()
    K = sp.csr_matrix((A.tangent(), cols, rowptr), shape=(A.ndof, A.ndof))
    b = np.random.default_rng(3).standard_normal(A.ndof)
    x = np.zeros(A.ndof)
    its, rn = A.ksp_solve(b, x, ksp_rtol=1e-10, ksp_restart=200, ksp_max_it=20000)
    xs = spl.spsolve(K.tocsc(), b)
    assert np.linalg.norm(K @ x - b) <= 1e-9 * np.linalg.norm(b)
    assert rel(x, xs) <= 1e-6


@pytest.mark.parametrize("law", [po.LAW_LINGRAD, po.LAW_GRADELASTTIME])
def test_newton_cgs2_matches_mgs(law):
    """Graph GMRES with classical Gram-Schmidt applied twice (two block passes
    per Arnoldi step) converges like the reference's modified Gram-Schmidt:
    the same Newton solution to the tolerance, and GMRES iteration counts
    within a few of each other."""
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(12, 3, 3), L=(4.0, 1.0, 1.0), law=law, bc_type=bct, neumann=neu)
    if law == po.LAW_GRADELASTTIME:
        par = prob.params()
        par[5], par[7] = 1.0, 1e-2
        prob.par = par
    out = {}
    for orth in (0, 1):
        A = gpu_case(prob)
        if prob.torder:
            A.set_state(np.zeros((3, A.ndof)))
        U = np.zeros(A.ndof)
        st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-8, ksp_restart=60, ksp_max_it=20000, orth=orth)
        assert st["converged"] == 1, st
        out[orth] = (U, st)
        A.close()
    assert rel(out[1][0], out[0][0]) <= 1e-7
    k0, k1 = out[0][1]["ksp_its_total"], out[1][1]["ksp_its_total"]
    assert abs(k1 - k0) <= max(3, 0.05 * k0), (k0, k1)


def test_newton_linear_beam_matches_direct_solve():
    """Config-1 style: clamped beam, tip traction, linear law; Newton-GMRES on
    the device converges and agrees with a direct CPU solve."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(16, 4, 4), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    A = gpu_case(prob)
    U = np.zeros(A.ndof)
    st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-10, ksp_restart=300, ksp_max_it=50000)
    assert st["converged"] == 1, st
    orc = po.OracleCase(prob)
    R0 = orc.residual(np.zeros((1, A.ndof)))
    rowptr, cols = orc.pattern()
    K = sp.csr_matrix((orc.tangent(np.zeros((1, A.ndof))), cols, rowptr), shape=(A.ndof, A.ndof))
    Us = spl.spsolve(K.tocsc(), -R0)
    assert rel(U, Us) <= 1e-7
    assert np.linalg.norm(orc.residual(U[None, :])) <= 1e-9


@pytest.mark.parametrize("precompute", ["0", "1"])
def test_geometry_cache_on_off_identical(precompute, monkeypatch):
    """The state-independent geometry cache gives bit-identical assembly when
    the law is evaluated inside the colour launches; with the law evaluated
    beforehand (a thread per point, which needs the cache; without the cache
    a warp per point) the two agree to round-off."""
    prob = po.Problem(nelem=(5, 3, 4), law=po.LAW_GRADELASTTIME, perturb=False)
    U = po.random_state(prob, 12)
    monkeypatch.setenv("IGAPGPU_LAW_PRECOMPUTE", precompute)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("IGAPGPU_GEOMETRY_CACHE", flag)
        A = gpu_case(prob)
        A.set_state(U)
        out.append((A.residual(), A.tangent()))
        A.close()
    if precompute == "0":
        np.testing.assert_array_equal(out[0][0], out[1][0])
        np.testing.assert_array_equal(out[0][1], out[1][1])
    else:
        assert rel(out[0][0], out[1][0]) <= 1e-13
        assert rel(out[0][1], out[1][1]) <= 1e-13


def test_norm2_matches_numpy():
    prob = po.Problem(nelem=(6, 3, 3), law=po.LAW_GRADELAST)
    A = gpu_case(prob)
    x = np.random.default_rng(9).standard_normal(A.ndof)
    assert abs(A.norm2(x) - np.linalg.norm(x)) <= 1e-14 * np.linalg.norm(x)


def test_unknown_law_is_an_error():
    knots, w, X = ig.beam_mesh((2, 2, 2))
    with pytest.raises(ig.IgapGpuError):
        ig.Assembly((2, 2, 2), knots, w, X, law=7)


def test_bad_sizes_are_errors():
    knots, w, X = ig.beam_mesh((2, 2, 2))
    with pytest.raises(ig.IgapGpuError):
        ig.Assembly((1, 2, 2), [np.zeros(6)] + knots[1:], w, X)
    with pytest.raises(ig.IgapGpuError):
        ig.Assembly((2, 2, 2), knots, w, X, nquad=9)


@pytest.mark.parametrize("prec", [ig.PREC_FP64, ig.PREC_SPLIT])
def test_newton_with_graphs_matches_without(prec):
    """Graph-replayed Newton step (captured assembly + device-resident GMRES
    cycles) gives the same iterates as the step-by-step path."""
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(12, 3, 3), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    knots, w, X = ig.beam_mesh(prob.nelem, prob.L)
    res = []
    for graphs in (0, 1):
        A = ig.Assembly(prob.nelem, knots, w, X, law=prob.law, par=prob.params(), bc_type=bct, neumann=neu)
        A.set_precision(prec)
        U = np.zeros(A.ndof)
        st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-10, ksp_restart=40, ksp_max_it=40000,
                     snes_max_it=15, use_graphs=graphs)
        res.append((U, st))
        A.close()
    (U0, s0), (U1, s1) = res
    assert s0["converged"] == 1 and s1["converged"] == 1, (s0, s1)
    assert np.linalg.norm(U1 - U0) <= 1e-8 * np.linalg.norm(U0)
    assert s1["newton_its"] == s0["newton_its"]


def test_dirichlet_rows_match_reference_tangent():
    """The Dirichlet rows the context reports are exactly the rows the
    reference's tangent reduced to identity rows (MatZeroRowsColumns), and
    impose_dirichlet writes g there and nothing elsewhere."""
    g = load("g_static_2x2x2")
    A = gpu_case(problem_from_golden(g))
    rows, vals = A.dirichlet()
    rowptr, cols, v = g["rowptr"], g["cols"], g["vals"]
    ident = []
    for r in range(len(rowptr) - 1):
        c, x = cols[rowptr[r]:rowptr[r + 1]], v[rowptr[r]:rowptr[r + 1]]
        if np.all(x[c != r] == 0.0) and np.all(x[c == r] == 1.0):
            ident.append(r)
    np.testing.assert_array_equal(np.sort(rows), np.array(ident))
    U = np.random.default_rng(3).standard_normal(A.ndof)
    V = A.impose_dirichlet(U.copy())
    np.testing.assert_array_equal(V[rows], vals)
    keep = np.ones(A.ndof, bool)
    keep[rows] = False
    np.testing.assert_array_equal(V[keep], U[keep])
    RR = A.residual(V)
    assert np.all(RR[rows] == 0.0)


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME])
def test_law_at_every_point_identical(law, monkeypatch):
    """Nonlinear laws are evaluated for every point in one launch before the
    colour launches (a thread per point, the measure sparsity fixed at compile
    time); the FP64 assembly agrees to round-off with that step turned off
    (the law evaluated a warp per point inside the colour launches, another
    summation order) and with the oracle, and the split tangent agrees within
    the split bound (with the step on, the split tangent's law runs in FP32
    arithmetic, without it the law is FP64)."""
    prob = po.Problem(nelem=(5, 3, 4), law=law, perturb=True)
    U = po.random_state(prob, 21)
    out = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("IGAPGPU_LAW_PRECOMPUTE", flag)
        A = gpu_case(prob)
        A.set_state(U)
        R, K = A.residual(), A.tangent()
        A.set_precision(ig.PREC_SPLIT)
        out[flag] = (R, K, A.tangent())
        A.close()
    assert rel(out["1"][0], out["0"][0]) <= 1e-13
    assert rel(out["1"][1], out["0"][1]) <= 1e-13
    assert rel(out["1"][2], out["0"][2]) <= 1e-5
    orc = po.OracleCase(prob)
    assert rel(out["1"][0], orc.residual(U)) <= 1e-12
    assert rel(out["1"][1], orc.tangent(U)) <= 1e-12


@pytest.mark.parametrize("name", ["g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2",
                                  "g_static_beamtest_4x4x4", "g_lingrad_8x2x2"])
def test_density_integral_vs_reference(name):
    """igapgpu_density against the reference's iga_intdensity (golden HH):
    energies, stresses, sector fractions, volume, traction work."""
    g = load(name)
    A = gpu_case(problem_from_golden(g))
    A.set_state(g["U"])
    HH = A.density()
    assert HH.shape == g["HH"].shape
    np.testing.assert_allclose(HH, g["HH"], rtol=1e-12, atol=1e-12 * np.abs(g["HH"]).max())


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME])
def test_solution_file_round_trip(law, tmp_path):
    """save_solution writes the reference's solution file (raw FP64 levels in
    DOF order, pinned against the reference's writer in test_oracle.py);
    load_solution reads it back, also from a file written by numpy."""
    prob = po.Problem(nelem=(3, 2, 2), law=law)
    A = gpu_case(prob)
    U = po.random_state(prob, 31)
    A.set_state(U)
    f = tmp_path / "U.bin"
    A.save_solution(str(f))
    raw = np.fromfile(f, dtype="<f8")
    exp = U[0] if A.torder == 0 else U[1:].ravel()
    np.testing.assert_array_equal(raw, exp)
    A.set_state(np.zeros_like(U))
    g = tmp_path / "V.bin"
    V = np.random.default_rng(32).standard_normal(exp.size)
    V.astype("<f8").tofile(g)
    A.load_solution(str(g))
    levels = V.reshape(-1, A.ndof)
    if A.torder == 0:
        np.testing.assert_array_equal(A.get_history(0), levels[0])
    else:
        for lvl in range(1, A.torder + 1):
            np.testing.assert_array_equal(A.get_history(lvl), levels[lvl - 1])
        np.testing.assert_array_equal(A.get_history(0), levels[0])
    with pytest.raises(ig.IgapGpuError):
        A.load_solution(str(tmp_path / "missing.bin"))


def test_point_block_jacobi_gmres():
    """GMRES with 3x3 point-block Jacobi (pc=2) and with the 2x2x2-cell block
    Jacobi (pc=3, blocks up to 24x24, clipped cells at the far faces: 8x3x2
    elements give 10x5x4 control points) solves the linear beam to the direct
    solution, in the host-driven and the graph-replayed cycles; point blocks
    take no more iterations than scalar Jacobi, cell blocks fewer than point
    blocks."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(8, 3, 2), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, perturb=True, bc_type=bct,
                      neumann=neu)
    A = gpu_case(prob)
    A.tangent_internal(np.zeros(A.ndof))
    rowptr, cols = A.pattern()
    K = sp.csr_matrix((A.tangent(), cols, rowptr), shape=(A.ndof, A.ndof))
    b = np.random.default_rng(4).standard_normal(A.ndof)
    xs = spl.spsolve(K.tocsc(), b)
    its = {}
    for pc in (1, 2, 3):
        for graphs in (0, 1):
            x = np.zeros(A.ndof)
            n, rn = A.ksp_solve(b, x, ksp_rtol=1e-10, ksp_restart=200, ksp_max_it=40000, pc=pc,
                                use_graphs=graphs)
            assert np.linalg.norm(K @ x - b) <= 1e-9 * np.linalg.norm(b)
            assert rel(x, xs) <= 1e-6
            its[(pc, graphs)] = n
    assert its[(2, 0)] == its[(2, 1)] and its[(3, 0)] == its[(3, 1)]
    assert its[(2, 0)] <= its[(1, 0)], its
    assert its[(3, 0)] < its[(2, 0)], its


def test_cell_block_jacobi_newton_static_law():
    """The static gradient law (indefinite tangents): Newton-GMRES with
    cell-block Jacobi reaches the residual tolerance, as with point-block
    Jacobi (measured on this 6x3x3 beam: 12,275 Krylov iterations against
    6,810 -- larger blocks of an indefinite tangent do not help here); a batch
    context refuses pc=3."""
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(6, 3, 3), L=(2.0, 1.0, 1.0), law=po.LAW_GRADELAST, perturb=True, bc_type=bct,
                      neumann=neu)
    kits = {}
    for pc in (2, 3):
        A = gpu_case(prob)
        U = np.zeros(A.ndof)
        st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-8, ksp_restart=100, ksp_max_it=100000, snes_max_it=20,
                     pc=pc, use_graphs=1)
        assert st["converged"] == 1, st
        assert np.linalg.norm(A.residual(U.copy())) <= 1e-10
        kits[pc] = st["ksp_its_total"]
        A.close()
    assert kits[2] > 0 and kits[3] > 0, kits
    insts = [dict(nelem=(3, 2, 2), knots=k, w=w, X=X, par=(1, 1, 0.1, 0, 0, 0, 0, 0, 0), bc_type=bct, neumann=neu)
             for (k, w, X) in [ig.beam_mesh((3, 2, 2), (2.0, 1.0, 1.0))]]
    B = ig.BatchAssembly(insts, law=ig.LAW_LINGRAD)
    with pytest.raises(ig.IgapGpuError):
        B.solve(np.zeros(B.ndof), pc=3, use_graphs=0)


@pytest.mark.parametrize("use_graphs", [0, 1])
def test_additive_schwarz_solves(use_graphs):
    """Restricted additive Schwarz (pc=4: the cells of pc=3 extended by one
    control-point layer, FP32 subdomain solves): GMRES on the linear beam
    reaches the direct-solve answer in fewer iterations than Jacobi, through
    the host-driven and the graph GMRES."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(16, 4, 4), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, bc_type=bct, neumann=neu)
    A = gpu_case(prob)
    A.tangent_internal(np.zeros(A.ndof))
    rowptr, cols = A.pattern()
    K = sp.csr_matrix((A.tangent(), cols, rowptr), shape=(A.ndof, A.ndof))
    b = np.random.default_rng(4).standard_normal(A.ndof)
    its = {}
    for pc in (1, 4):
        x = np.zeros(A.ndof)
        U = np.zeros(A.ndof)
        if use_graphs:
            st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-10, ksp_restart=200, ksp_max_it=50000, pc=pc,
                         use_graphs=1)
            assert st["converged"] == 1, st
            its[pc] = st["ksp_its_total"]
        else:
            its[pc], _ = A.ksp_solve(b, x, ksp_rtol=1e-10, ksp_restart=200, ksp_max_it=50000, pc=pc)
            assert np.linalg.norm(K @ x - b) <= 1e-9 * np.linalg.norm(b)
            assert rel(x, spl.spsolve(K.tocsc(), b)) <= 1e-6
    print("GMRES iterations, Jacobi vs additive Schwarz:", its)
    assert its[4] < its[1], its


def test_additive_schwarz_transient_law():
    """pc=4 on one transient step of the reference's three-level law (12x3x3,
    density 1, dt 1e-2): Newton reaches the tolerance with fewer GMRES
    iterations than with Jacobi.  (On the indefinite static law the FP32
    subdomain solves of indefinite blocks make GMRES stagnate; point-block
    Jacobi is the preconditioner for that law.)"""
    bct, neu = po.clamp_bc((0,), 1, (0, 0, -1e-3))
    prob = po.Problem(nelem=(12, 3, 3), L=(4.0, 1.0, 1.0), law=po.LAW_GRADELASTTIME, bc_type=bct, neumann=neu)
    par = prob.params()
    par[5], par[7] = 1.0, 1e-2
    prob.par = par
    kits = {}
    for pc in (1, 4):
        A = gpu_case(prob)
        A.set_state(np.zeros((3, A.ndof)))
        U = np.zeros(A.ndof)
        st = A.solve(U, snes_abstol=1e-10, ksp_rtol=1e-8, ksp_restart=100, ksp_max_it=100000, pc=pc, use_graphs=1,
                     orth=1)
        assert st["converged"] == 1, st
        kits[pc] = st["ksp_its_total"]
        A.close()
    print("GMRES iterations, Jacobi vs additive Schwarz:", kits)
    assert kits[4] < kits[1], kits


def field_close(F, G, tol=1e-12):
    """Per field column: |F - G| <= tol * max |G| of that column."""
    scale = np.maximum(np.abs(G).reshape(-1, G.shape[-1]).max(axis=0), 1e-300)
    return np.all(np.abs(F - G) <= tol * scale)


@pytest.mark.parametrize("name", ["g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2"])
def test_field_sampling_vs_reference(name):
    """igapgpu_sample_field against the reference's basis, inverse and field
    callbacks on the plot lattice of iga_plotfield (golden field): knot
    coordinates bit-exact, positions to round-off, fields to 1e-12 of each
    column's scale, sector codes exact."""
    g = load(name)
    A = gpu_case(problem_from_golden(g))
    A.set_state(float(g["field_scale"]) * g["U"])
    F, xq, X = A.sample_field(int(g["field_nppe"]))
    assert F.shape == g["field"].shape
    np.testing.assert_array_equal(xq, g["field_xq"])
    np.testing.assert_allclose(X, g["field_X"], rtol=0, atol=1e-14)
    assert field_close(F, g["field"])
    if int(g["law"]) != po.LAW_LINGRAD:
        np.testing.assert_array_equal(F[..., -1], g["field"][..., -1])


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME, po.LAW_LINGRAD])
def test_field_sampling_vs_oracle_device_buffers(law):
    """Perturbed geometry, nppe = 3, against the restatement; outputs written
    straight into device buffers match the host-buffer path bit for bit."""
    torch = pytest.importorskip("torch")
    import ctypes
    prob = po.Problem(nelem=(5, 3, 4), L=(2.0, 1.0, 1.5), law=law, perturb=True)
    U = 20.0 * po.random_state(prob, 41)
    A = gpu_case(prob)
    A.set_state(U)
    F, xq, X = A.sample_field(3)
    Fo, xo, Xo = po.OracleCase(prob).field(U, 3)
    np.testing.assert_array_equal(xq, xo)
    np.testing.assert_allclose(X, Xo, rtol=0, atol=1e-14)
    assert field_close(F, Fo)
    dF = torch.zeros(F.shape, dtype=torch.float64, device="cuda")
    dX = torch.zeros(X.shape, dtype=torch.float64, device="cuda")
    rc = ig.lib().igapgpu_sample_field(A.h, 3, ctypes.c_void_p(dF.data_ptr()), None,
                                       ctypes.c_void_p(dX.data_ptr()), None, None)
    assert rc == 0
    np.testing.assert_array_equal(dF.cpu().numpy(), F)
    np.testing.assert_array_equal(dX.cpu().numpy(), X)
    with pytest.raises(ig.IgapGpuError):
        A.sample_field(0)


def test_colour_scatter_has_no_lost_updates():
    """Race check of the colour-partitioned scatter on the GPU: with a plain
    read-modify-write per slot, colour by colour, every CSR slot ends at the
    number of elements whose support holds both of its control points."""
    from slot_counts import explicit_counts

    for nelem in ((5, 4, 3), (7, 3, 4)):
        A = gpu_case(po.Problem(nelem=nelem, law=po.LAW_LINGRAD, perturb=True))
        rowptr, cols = A.pattern()
        np.testing.assert_array_equal(A.debug_slot_counts(), explicit_counts(nelem, rowptr, cols))
        A.close()

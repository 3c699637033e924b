"""CPU oracle checks (no GPU).

The project's C restatement (oracle/liborc.so) is pinned
  * against the reference's own compiled code (oracle/_ref) where it exists,
  * and against golden vectors generated from the reference
    (tests/golden/make_golden.py), which travel with the repository.
"""
import ctypes
import math
import os

import numpy as np
import pytest

import pyoracle as po
from conftest import GOLDEN

needs_ref = pytest.mark.skipif(not po.ref_available(), reason="reference not compiled here")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def problem_from_golden(g):
    return po.Problem(nelem=tuple(int(x) for x in g["nelem"]), L=tuple(g["L"]), law=int(g["law"]),
                      perturb=bool(g["perturb"]), par=g["par"], bc_type=g["bc_type"].astype(np.int32),
                      neumann=g["neumann"])


# ------------------------------------------------------------- quadrature
def test_gauss_legendre_closed_form():
    x, w = po.gauss_legendre(4)
    a = math.sqrt(3 / 7 - 2 / 7 * math.sqrt(6 / 5))
    b = math.sqrt(3 / 7 + 2 / 7 * math.sqrt(6 / 5))
    xe = [(1 - b) / 2, (1 - a) / 2, (1 + a) / 2, (1 + b) / 2]
    we = [(18 - math.sqrt(30)) / 72, (18 + math.sqrt(30)) / 72] * 1
    we = [we[0], we[1], we[1], we[0]]
    np.testing.assert_allclose(x, xe, rtol=0, atol=2e-16)
    np.testing.assert_allclose(w, we, rtol=0, atol=2e-16)


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6])
def test_gauss_legendre_golden(n):
    g = load("quadrature")
    x, w = po.gauss_legendre(n)
    np.testing.assert_allclose(x, g[f"x{n}"], rtol=0, atol=4e-16)
    np.testing.assert_allclose(w, g[f"w{n}"], rtol=0, atol=4e-16)


# ------------------------------------------------------------------ laws
@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME, po.LAW_LINGRAD])
def test_law_golden(law):
    g = load("laws")
    mask = np.ones(30, bool)
    mask[[0, 10, 20]] = False
    for u, rr_ref, tt_ref in zip(g[f"u_{law}"], g[f"rr_{law}"], g[f"tt_{law}"]):
        rr, tt = po.law_eval("orc", law, u, g[f"par_{law}"])
        # elastic entries and value (inertia) entries scaled separately
        assert np.abs(rr - rr_ref)[mask].max() <= 1e-13 * max(np.abs(rr_ref[mask]).max(), 1e-300)
        assert np.abs(rr - rr_ref)[~mask].max() <= 1e-13 * max(np.abs(rr_ref[~mask]).max(), 1.0)
        e = np.abs(tt - tt_ref)[np.ix_(mask, mask)].max()
        assert e <= 1e-13 * np.abs(tt_ref[np.ix_(mask, mask)]).max()
        np.testing.assert_allclose(tt[~mask][:, ~mask], tt_ref[~mask][:, ~mask], rtol=1e-14)


@pytest.mark.parametrize("law", [po.LAW_GRADELAST, po.LAW_GRADELASTTIME, po.LAW_LINGRAD])
def test_law_tangent_is_jacobian_and_symmetric(law):
    par = po.Problem(law=law).params()
    rng = np.random.default_rng(3)
    u = rng.uniform(-0.05, 0.05, 90)
    rr, tt = po.law_eval("orc", law, u, par)
    h = 1e-6
    fd = np.zeros((30, 30))
    for j in range(30):
        up = u.copy(); up[j] += h
        um = u.copy(); um[j] -= h
        fd[:, j] = (po.law_eval("orc", law, up, par)[0] - po.law_eval("orc", law, um, par)[0]) / (2 * h)
    assert np.abs(fd - tt).max() <= 1e-7 * np.abs(tt).max()
    assert np.abs(tt - tt.T).max() <= 1e-14 * np.abs(tt).max()


def test_gradelast_undeformed_is_unstable():
    """At the default r=0.25, curv=0.5 the quadratic Landau coefficient is
    negative (phys/gradelast.c:47), so the undeformed tangent is indefinite."""
    lib = po.orc()
    par = po.Problem(law=po.LAW_GRADELAST).params()
    rr, tt = po.law_eval("orc", po.LAW_GRADELAST, np.zeros(90), par)
    assert np.abs(rr).max() == 0.0
    ev = np.linalg.eigvalsh(tt)
    assert ev.min() < 0 < ev.max()


# ------------------------------------------------------------- assembly
@pytest.mark.parametrize("name", ["g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2"])
def test_assembly_full_golden(name):
    g = load(name)
    prob = problem_from_golden(g)
    case = po.OracleCase(prob)
    U = g["U"]
    RR = case.residual(U)
    assert np.linalg.norm(RR - g["RR"]) <= 1e-13 * np.linalg.norm(g["RR"])
    rowptr, cols = case.pattern()
    np.testing.assert_array_equal(rowptr, g["rowptr"])
    np.testing.assert_array_equal(cols, g["cols"])
    vals = case.tangent(U)
    assert np.linalg.norm(vals - g["vals"]) <= 1e-13 * np.linalg.norm(g["vals"])


@pytest.mark.parametrize("name", ["g_static_beamtest_4x4x4", "g_lingrad_8x2x2"])
def test_assembly_summary_golden(name):
    g = load(name)
    prob = problem_from_golden(g)
    case = po.OracleCase(prob)
    U = g["U"]
    RR = case.residual(U)
    assert np.linalg.norm(RR - g["RR"]) <= 1e-13 * np.linalg.norm(g["RR"])
    rowptr, cols = case.pattern()
    np.testing.assert_array_equal(rowptr, g["rowptr"])
    assert cols.astype(np.int64).sum() == g["cols_sum"]
    assert (cols.astype(np.int64) * np.arange(len(cols)) % 1000003).sum() == g["cols_wsum"]
    vals = case.tangent(U)
    assert abs(np.linalg.norm(vals) - g["vals_norm"]) <= 1e-13 * g["vals_norm"]
    np.testing.assert_allclose(vals[g["sample_idx"]], g["sample_vals"], rtol=0,
                               atol=1e-13 * np.abs(g["sample_vals"]).max())


def test_sanity_value_glibc_rand():
    """4x4x4 unit cube, static law, face x=0 clamped (both orders), U from
    glibc rand() seed 123456 scaled 0.01 on every DOF (IGAPSolvRand,
    src/interface.c:261-269): the reference gives |R|^2 = 3.68958470382283..."""
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("glibc not available")
    bct, neu = po.clamp_bc((0,))
    prob = po.Problem(nelem=(4, 4, 4), law=po.LAW_GRADELAST, bc_type=bct, neumann=neu)
    libc.srand(123456)
    U = np.array([0.01 * ((libc.rand() % 999999999) / 999999999.0) for _ in range(prob.ndof)])
    RR = po.OracleCase(prob).residual(U[None, :])
    assert abs((RR ** 2).sum() - 3.68958470382283) <= 1e-13


def test_partition_of_unity_and_numbering():
    """sum_b R_b = 1 implies a rigid translation gives zero volume residual for
    the static law; DOF numbering 3*((ny+2)(nz+2) ix + (nz+2) iy + iz) + d
    (src/interface.c:163-168) is the CSR row order."""
    prob = po.Problem(nelem=(3, 2, 2), law=po.LAW_GRADELAST)
    case = po.OracleCase(prob)
    U = np.tile([0.3, -0.2, 0.1], prob.ndof // 3)[None, :]
    RR = case.residual(U)
    assert np.abs(RR).max() < 1e-12
    rowptr, cols = case.pattern()
    nb = prob.nbasis
    # row of control point (ix,iy,iz), dof d has the diagonal column equal to itself
    for ix, iy, iz, d in [(0, 0, 0, 0), (4, 3, 2, 2), (2, 1, 3, 1)]:
        r = 3 * (nb[1] * nb[2] * ix + nb[2] * iy + iz) + d
        assert r in cols[rowptr[r]:rowptr[r + 1]]


# ---------------------------------------------- against the live reference
@needs_ref
@pytest.mark.parametrize("law,perturb,nelem", [
    (po.LAW_GRADELAST, False, (3, 2, 4)),
    (po.LAW_GRADELAST, True, (4, 4, 4)),
    (po.LAW_LINGRAD, False, (5, 2, 3)),
    (po.LAW_GRADELASTTIME, False, (2, 3, 2)),
])
def test_assembly_vs_reference(law, perturb, nelem):
    bct, neu = po.clamp_bc((0, 3), 5, (1e-3, 2e-3, -1e-3))
    bct[6 * 1 + 3:6 * 1 + 6] = 1
    neu[6 * 1 + 4] = 5e-4  # high-order traction on face 1, dof 1
    prob = po.Problem(nelem=nelem, law=law, perturb=perturb, bc_type=bct, neumann=neu,
                      par_dirichlet=np.linspace(0.01, 0.09, 9))
    U = po.random_state(prob, 17)
    ref = po.RefCase(prob)
    orc = po.OracleCase(prob)
    R1 = ref.residual(U)
    R2 = orc.residual(U)
    assert np.linalg.norm(R1 - R2) <= 1e-13 * np.linalg.norm(R1)
    rp, cols, v1 = ref.tangent(U)
    rp2, cols2 = orc.pattern()
    np.testing.assert_array_equal(rp, rp2)
    np.testing.assert_array_equal(cols, cols2)
    v2 = orc.tangent(U)
    assert np.linalg.norm(v1 - v2) <= 1e-13 * np.linalg.norm(v1)


@needs_ref
def test_per_direction_mesh_equals_reference_igabeam():
    """The per-direction beam constructor reproduces MeshIGABeam
    (mesh/igabeam.c) and MeshIGABeamTest bit for bit when every direction has
    2^mref elements."""
    for perturb, kind in ((False, po.RefCase.MESH_REF_IGABEAM), (True, po.RefCase.MESH_REF_IGABEAMTEST)):
        prob = po.Problem(nelem=(8, 8, 8), perturb=perturb)
        a = po.RefCase(prob, mesh_kind=kind).mesh()
        knots, w, X = po.mesh_beam(prob)
        np.testing.assert_array_equal(a[3], knots)
        np.testing.assert_array_equal(a[4], w)
        np.testing.assert_array_equal(a[5], X)


@needs_ref
def test_global_idx_identity_on_one_rank():
    prob = po.Problem(nelem=(3, 2, 2))
    g = po.RefCase(prob).global_idx()
    np.testing.assert_array_equal(g, np.arange(prob.ndof))


@pytest.mark.skipif(not po.ref_available(), reason="needs oracle/_ref (reference sources)")
def test_reference_density_volume_known_answer():
    """The reference's density integral: its volume density integrates to the
    volume of the beam geometry, L_d (1 + 1/n_d) per direction for the
    control-net formula of mesh/igabeam.c:68-70."""
    for law, nelem, L in ((po.LAW_GRADELASTTIME, (3, 2, 2), (1.0, 1.0, 1.0)),
                          (po.LAW_LINGRAD, (4, 2, 3), (4.0, 1.0, 1.0))):
        prob = po.Problem(nelem=nelem, L=L, law=law)
        HH = po.RefCase(prob).density(po.random_state(prob, 5))
        vol = np.prod([l * (1.0 + 1.0 / n) for l, n in zip(L, nelem)])
        assert abs(HH[1] - vol) <= 1e-12 * vol


def test_golden_densities_present():
    for name in ("g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2"):
        g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
        assert "HH" in g.files and np.all(np.isfinite(g["HH"]))


@pytest.mark.skipif(not po.ref_available(), reason="needs oracle/_ref (reference sources)")
def test_reference_solution_file_layout(tmp_path):
    """The reference's solution file (IGAPSolvSaveSolution) is the raw FP64
    history levels in DOF order: level 0 for a static law, levels 1..torder
    for the transient law; its reader restores them (level 0 = level 1)."""
    for law, nelem in ((po.LAW_GRADELAST, (3, 2, 2)), (po.LAW_GRADELASTTIME, (2, 3, 2))):
        prob = po.Problem(nelem=nelem, law=law)
        rc = po.RefCase(prob)
        U = po.random_state(prob, 9)
        rc.set_state(U)
        f = str(tmp_path / f"U_{law}.bin")
        rc.save(f)
        raw = np.fromfile(f, dtype="<f8")
        levels = U.reshape(-1, rc.ndof)
        exp = levels[0] if law == po.LAW_GRADELAST else levels[1:].ravel()
        np.testing.assert_array_equal(raw, exp)
        rc.set_state(np.zeros_like(U))
        rc.load(f)
        got = np.zeros_like(U)
        po.ref().ref_case_get_state(rc.h, got.ctypes.data)
        got = got.reshape(-1, rc.ndof)
        if law == po.LAW_GRADELAST:
            np.testing.assert_array_equal(got[0], levels[0])
        else:
            np.testing.assert_array_equal(got[1:], levels[1:])
            np.testing.assert_array_equal(got[0], levels[1])


# ----------------------------------------------------------- field sampling
FIELD_CASES = ("g_static_2x2x2", "g_lingrad_4x2x2", "g_transient_3x2x2")


def field_close(F, G, tol=1e-12):
    """Per field column: |F - G| <= tol * max |G| of that column (sector codes exact)."""
    scale = np.maximum(np.abs(G).reshape(-1, G.shape[-1]).max(axis=0), 1e-300)
    return np.all(np.abs(F - G) <= tol * scale)


@pytest.mark.parametrize("name", FIELD_CASES)
def test_field_sampling_golden(name):
    """The restated plot loop with the restated basis and field callbacks
    (liborc) against the reference's basis, inverse and field callbacks
    (golden field at field_scale x the state, plot lattice of nppe = 2)."""
    g = load(name)
    prob = problem_from_golden(g)
    F, xq, X = po.OracleCase(prob).field(float(g["field_scale"]) * g["U"], int(g["field_nppe"]))
    assert F.shape == g["field"].shape
    np.testing.assert_array_equal(xq, g["field_xq"])
    np.testing.assert_allclose(X, g["field_X"], rtol=0, atol=1e-14)
    assert field_close(F, g["field"])
    if prob.law != po.LAW_LINGRAD:  # sector codes: exact, and more than one occurs
        np.testing.assert_array_equal(F[..., -1], g["field"][..., -1])
        assert len(np.unique(g["field"][..., -1])) > 1


@needs_ref
@pytest.mark.parametrize("law,perturb", [(po.LAW_GRADELAST, True), (po.LAW_GRADELASTTIME, False),
                                         (po.LAW_LINGRAD, True)])
def test_field_sampling_vs_reference_callbacks(law, perturb):
    prob = po.Problem(nelem=(3, 2, 4), L=(2.0, 1.0, 1.5), law=law, perturb=perturb)
    U = 20.0 * po.random_state(prob, 31)
    Fr, xr, Xr = po.RefCase(prob).field(U, 3)
    Fo, xo, Xo = po.OracleCase(prob).field(U, 3)
    np.testing.assert_array_equal(xo, xr)
    np.testing.assert_allclose(Xo, Xr, rtol=0, atol=1e-14)
    assert field_close(Fo, Fr)


def test_field_sampling_linear_state_known_answer():
    """A state linear in the control-point positions, U_b = A x_b, is
    reproduced exactly by the (unit-weight) spline space: the sampled value is
    A x at the sample position, the gradient A, the Hessian 0; the lattice
    points sit 1e-15 inside the element spans."""
    prob = po.Problem(nelem=(4, 2, 3), L=(4.0, 1.0, 1.0), law=po.LAW_LINGRAD, perturb=True)
    _, _, Xc = po.mesh_beam(prob)
    A = np.array([[1e-3, 2e-3, -1e-3], [0.5e-3, -1e-3, 3e-3], [2e-3, 1e-3, 1e-3]])
    U = (Xc.reshape(-1, 3) @ A.T).reshape(1, -1)
    F, xq, X = po.OracleCase(prob).field(U, 2)
    u = F[..., :30].reshape(F.shape[:3] + (3, 10))
    np.testing.assert_allclose(u[..., 0], X @ A.T, rtol=0, atol=1e-15)
    np.testing.assert_allclose(u[..., 1:4], np.broadcast_to(A, u.shape[:3] + (3, 3)), rtol=0, atol=1e-13)
    assert np.abs(u[..., 4:]).max() <= 1e-12
    k0, k1 = 0.75, 1.0  # last knot span in x
    assert xq[0, 0, 0, 0] == 1e-15
    assert xq[-1, 0, 0, 0] == k0 + 1e-15 + (k1 - k0) * 2 / 2 - 2 * 1e-15 * 1 and xq[-1, 0, 0, 0] < 1.0


def test_slot_multiplicity_formula():
    """The expected CSR slot multiplicities of the scatter race check: the
    closed form equals an explicit element loop over the oracle's pattern, and
    every slot of the full-stencil pattern is touched by at least one element."""
    from slot_counts import explicit_counts, formula_counts

    for nelem in ((3, 2, 2), (5, 4, 3), (1, 1, 2)):
        case = po.OracleCase(po.Problem(nelem=nelem, law=po.LAW_LINGRAD))
        rowptr, cols = case.pattern()
        ex = explicit_counts(nelem, rowptr, cols)
        np.testing.assert_array_equal(ex, formula_counts(nelem, rowptr, cols))
        assert ex.min() >= 1 and ex.max() == np.prod([min(3, n) for n in nelem])

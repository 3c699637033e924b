"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries:

* ``oracle/liborc.so`` -- the project's own C restatement of IGAP4's assembly
  path (``oracle/igap_oracle.c``); builds anywhere with gcc.
* ``oracle/_ref/libigapref.so`` -- the reference's own sources compiled
  unchanged against single-rank MPI/PETSc stand-ins (``oracle/build_ref.sh``);
  present only where the reference tree exists.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORC = os.path.join(HERE, "liborc.so")
LIBREF = os.path.join(HERE, "_ref", "libigapref.so")

LAW_GRADELAST, LAW_GRADELASTTIME, LAW_LINGRAD = 0, 1, 2
LAW_TORDER = {LAW_GRADELAST: 0, LAW_GRADELASTTIME: 2, LAW_LINGRAD: 0}

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_L = ctypes.POINTER(ctypes.c_long)


def _p(a, t=_D):
    return None if a is None else a.ctypes.data_as(t)


def _load(path):
    return ctypes.CDLL(path)


_orc = None
_ref = None


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(LIBORC):
            raise RuntimeError("oracle/liborc.so missing: run oracle/build_oracle.sh")
        _orc = _load(LIBORC)
        _orc.orc_case_create.restype = ctypes.c_void_p
        _orc.orc_case_nnz.restype = ctypes.c_long
        _orc.orc_evalN.restype = ctypes.c_double
        for f in ("orc_case_ndof", "orc_case_torder", "orc_case_nnz", "orc_case_destroy"):
            getattr(_orc, f).argtypes = [ctypes.c_void_p]
        for f in ("orc_case_pattern", "orc_case_residual", "orc_case_tangent"):
            getattr(_orc, f).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for f in ("orc_case_tangent_elements", "orc_case_residual_elements"):
            getattr(_orc, f).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_long, ctypes.c_long]
        _orc.orc_evalN.argtypes = [_D, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double]
        _orc.orc_gauss_legendre.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, _D]
        _orc.orc_case_field.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    return _orc


def ref_available() -> bool:
    return os.path.exists(LIBREF)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref/libigapref.so missing (reference tree not built here)")
        _ref = _load(LIBREF)
        _ref.ref_case_create.restype = ctypes.c_void_p
        _ref.ref_case_tangent.restype = ctypes.c_long
        _ref.ref_evalN.restype = ctypes.c_double
        for f in ("ref_case_ndof", "ref_case_torder", "ref_case_nlocal", "ref_case_destroy",
                  "ref_case_tangent"):
            getattr(_ref, f).argtypes = [ctypes.c_void_p]
        for f in ("ref_case_set_state", "ref_case_get_state", "ref_case_residual",
                  "ref_case_global_idx"):
            getattr(_ref, f).argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _ref.ref_case_tangent_csr.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 3
        _ref.ref_case_density.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _ref.ref_case_field.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
        _ref.ref_case_save.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _ref.ref_case_load.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        _ref.ref_case_mesh_info.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 3
        _ref.ref_case_mesh_arrays.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 3
        _ref.ref_gauss_legendre.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, _D, _D]
        _ref.ref_evalN.argtypes = [_D, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_double]
    return _ref


# --------------------------------------------------------------- problem spec
@dataclass
class Problem:
    """One assembly problem: beam mesh, law, boundary conditions."""

    nelem: tuple = (4, 4, 4)
    L: tuple = (1.0, 1.0, 1.0)
    p: int = 2
    perturb: bool = False
    law: int = LAW_GRADELAST
    par: np.ndarray | None = None
    nquad: int = 4
    bc_type: np.ndarray = field(default_factory=lambda: np.ones(36, np.int32))
    par_dirichlet: np.ndarray = field(default_factory=lambda: np.zeros(9))
    neumann: np.ndarray = field(default_factory=lambda: np.zeros(36))

    @property
    def torder(self):
        return LAW_TORDER[self.law]

    @property
    def nbasis(self):
        return tuple(n + self.p for n in self.nelem)

    @property
    def ndof(self):
        nb = self.nbasis
        return 3 * nb[0] * nb[1] * nb[2]

    def params(self):
        if self.par is not None:
            return np.ascontiguousarray(self.par, dtype=np.float64)
        par = np.zeros(9)
        orc().orc_law_default_par(self.law, _p(par))
        return par


def clamp_bc(faces=(0,), traction_face=None, traction=(0.0, 0.0, 0.0)):
    """bc_type/neumann tables: listed faces clamped (u = 0 and du/dn = 0, both
    orders), others traction-free, optional constant traction on one face.
    Table index: 6*face + 3*order + dof (src/assmcore_iga.c:331,367)."""
    bct = np.ones(36, np.int32)
    neu = np.zeros(36)
    for f in faces:
        bct[6 * f:6 * f + 6] = 0
    if traction_face is not None:
        for d in range(3):
            neu[6 * traction_face + d] = traction[d]
    return bct, neu


def mesh_beam(prob: Problem):
    nelem = np.array(prob.nelem, np.int32)
    L = np.array(prob.L, np.float64)
    nk = sum(n + 1 + 2 * prob.p for n in prob.nelem)
    ncp = int(np.prod(prob.nbasis))
    knots = np.zeros(nk)
    w = np.zeros(ncp)
    X = np.zeros(3 * ncp)
    orc().orc_mesh_beam(_p(nelem, _I), _p(L), prob.p, int(prob.perturb), _p(knots), _p(w), _p(X))
    return knots, w, X


def gauss_legendre(n, a=0.0, b=1.0):
    x = np.zeros(n)
    w = np.zeros(n)
    orc().orc_gauss_legendre(n, a, b, _p(x), _p(w))
    return x, w


def random_state(prob: Problem, seed: int, scale: float = 1e-2):
    """Seeded state, i.i.d. uniform in [-scale, scale] on every DOF and every
    history level: shape (torder+1, ndof)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-scale, scale, size=(prob.torder + 1, prob.ndof))


class OracleCase:
    """The project's C restatement."""

    def __init__(self, prob: Problem):
        self.prob = prob
        knots, w, X = mesh_beam(prob)
        nelem = np.array(prob.nelem, np.int32)
        self._keep = (knots, w, X)
        self.h = ctypes.c_void_p(orc().orc_case_create(
            _p(nelem, _I), prob.p, _p(knots), _p(w), _p(X), prob.law, _p(prob.params()),
            prob.nquad, _p(np.ascontiguousarray(prob.bc_type, np.int32), _I),
            _p(np.ascontiguousarray(prob.par_dirichlet, np.float64)),
            _p(np.ascontiguousarray(prob.neumann, np.float64))))
        self.ndof = orc().orc_case_ndof(self.h)
        self.nnz = orc().orc_case_nnz(self.h)

    def __del__(self):
        try:
            orc().orc_case_destroy(self.h)
        except Exception:
            pass

    def pattern(self):
        rowptr = np.zeros(self.ndof + 1, np.int64)
        cols = np.zeros(self.nnz, np.int32)
        orc().orc_case_pattern(self.h, rowptr.ctypes.data, cols.ctypes.data)
        return rowptr, cols

    def residual(self, U_hist):
        U = np.ascontiguousarray(U_hist, np.float64)
        RR = np.zeros(self.ndof)
        orc().orc_case_residual(self.h, U.ctypes.data, RR.ctypes.data)
        return RR

    def tangent(self, U_hist):
        U = np.ascontiguousarray(U_hist, np.float64)
        vals = np.zeros(self.nnz)
        orc().orc_case_tangent(self.h, U.ctypes.data, vals.ctypes.data)
        return vals

    def tangent_elements(self, U_hist, e0, e1):
        U = np.ascontiguousarray(U_hist, np.float64)
        vals = np.zeros(self.nnz)
        orc().orc_case_tangent_elements(self.h, U.ctypes.data, vals.ctypes.data, e0, e1)
        return vals

    def field(self, U_hist, nppe):
        """Field on the plot lattice: (field [NX,NY,NZ,nfield], xq, X [NX,NY,NZ,3])."""
        U = np.ascontiguousarray(U_hist, np.float64)
        shape = field_lattice(self.prob, nppe)
        nf = 6 if self.prob.law == LAW_GRADELASTTIME else 33
        F = np.zeros(shape + (nf,))
        xq = np.zeros(shape + (3,))
        X = np.zeros(shape + (3,))
        orc().orc_case_field(self.h, U.ctypes.data, int(nppe), F.ctypes.data, xq.ctypes.data, X.ctypes.data)
        return F, xq, X

    def residual_elements(self, U_hist, e0, e1):
        U = np.ascontiguousarray(U_hist, np.float64)
        RR = np.zeros(self.ndof)
        orc().orc_case_residual_elements(self.h, U.ctypes.data, RR.ctypes.data, e0, e1)
        return RR


class RefCase:
    """The reference's own code (oracle/_ref), set up through IGAPAssmInit."""

    MESH_BEAM, MESH_BEAMTEST, MESH_REF_IGABEAM, MESH_REF_IGABEAMTEST = 0, 1, 2, 3

    def __init__(self, prob: Problem, mesh_kind=None):
        self.prob = prob
        if mesh_kind is None:
            mesh_kind = self.MESH_BEAMTEST if prob.perturb else self.MESH_BEAM
        nelem = np.array(prob.nelem, np.int32)
        L = np.array(prob.L, np.float64)
        per = np.zeros(3, np.int32)
        par = prob.params() if prob.par is not None else None
        self.h = ctypes.c_void_p(ref().ref_case_create(
            _p(nelem, _I), _p(L), prob.p, _p(per, _I), mesh_kind, prob.law, _p(par),
            _p(np.ascontiguousarray(prob.bc_type, np.int32), _I),
            _p(np.ascontiguousarray(prob.par_dirichlet, np.float64)),
            _p(np.ascontiguousarray(prob.neumann, np.float64)), None))
        self.ndof = ref().ref_case_ndof(self.h)
        self.torder = ref().ref_case_torder(self.h)

    def set_state(self, U_hist):
        U = np.ascontiguousarray(U_hist, np.float64)
        assert U.size == (self.torder + 1) * self.ndof
        ref().ref_case_set_state(self.h, U.ctypes.data)

    def residual(self, U_hist):
        self.set_state(U_hist)
        RR = np.zeros(self.ndof)
        ref().ref_case_residual(self.h, RR.ctypes.data)
        return RR

    def save(self, fname):
        ref().ref_case_save(self.h, os.fsencode(fname))

    def load(self, fname):
        ref().ref_case_load(self.h, os.fsencode(fname))

    def density(self, U_hist):
        """iga_intdensity of the reference on this state (its densities)."""
        self.set_state(U_hist)
        HH = np.zeros(16)
        n = ref().ref_case_density(self.h, HH.ctypes.data)
        return HH[:n].copy()

    def field(self, U_hist, nppe):
        """The reference's basis, inverse and field callback on the plot
        lattice (restated loop): (field, xq, X) as OracleCase.field."""
        self.set_state(U_hist)
        shape = field_lattice(self.prob, nppe)
        nf = 6 if self.prob.law == LAW_GRADELASTTIME else 33
        F = np.zeros(shape + (nf,))
        xq = np.zeros(shape + (3,))
        X = np.zeros(shape + (3,))
        got = ref().ref_case_field(self.h, int(nppe), F.ctypes.data, xq.ctypes.data, X.ctypes.data)
        assert got == nf
        return F, xq, X

    def tangent(self, U_hist):
        self.set_state(U_hist)
        nnz = ref().ref_case_tangent(self.h)
        rowptr = np.zeros(self.ndof + 1, np.int64)
        cols = np.zeros(nnz, np.int32)
        vals = np.zeros(nnz)
        ref().ref_case_tangent_csr(self.h, rowptr.ctypes.data, cols.ctypes.data, vals.ctypes.data)
        return rowptr, cols, vals

    def global_idx(self):
        n = ref().ref_case_nlocal(self.h)
        g = np.zeros(n, np.int32)
        ref().ref_case_global_idx(self.h, g.ctypes.data)
        return g

    def mesh(self):
        nelem = np.zeros(3, np.int32)
        nknot = np.zeros(3, np.int32)
        nbasis = np.zeros(3, np.int32)
        ref().ref_case_mesh_info(self.h, nelem.ctypes.data, nknot.ctypes.data, nbasis.ctypes.data)
        p = self.prob.p
        ncp = int(np.prod(nelem + p))
        knots = np.zeros(int(nknot.sum()))
        w = np.zeros(ncp)
        X = np.zeros(3 * ncp)
        ref().ref_case_mesh_arrays(self.h, knots.ctypes.data, w.ctypes.data, X.ctypes.data)
        return nelem, nknot, nbasis, knots, w, X


def field_lattice(prob: Problem, nppe: int):
    """Plot lattice of iga_plotfield: nppe samples per element and direction
    plus the far faces."""
    return tuple(int(nppe) * int(n) + 1 for n in prob.nelem)


def law_eval(which, law, u, par):
    """Per-point law through the oracle ('orc') or the reference ('ref')."""
    lib = orc() if which == "orc" else ref()
    u = np.ascontiguousarray(u, np.float64)
    par = np.ascontiguousarray(par, np.float64)
    rr = np.zeros(30)
    tt = np.zeros(900)
    if which == "orc":
        lib.orc_law_residual(law, _p(rr), _p(u), _p(par))
        lib.orc_law_tangent(law, _p(tt), _p(u), _p(par))
    else:
        lib.ref_law_residual(law, _p(rr), _p(u), _p(par))
        lib.ref_law_tangent(law, _p(tt), _p(u), _p(par))
    return rr, tt.reshape(30, 30)


def csr_to_dense(rowptr, cols, vals, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, cols[rowptr[r]:rowptr[r + 1]]] = vals[rowptr[r]:rowptr[r + 1]]
    return A

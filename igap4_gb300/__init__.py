"""igap4_gb300 -- GB300-native element assembly and Newton-Krylov for IGAP4.

Python access to ``libigapgpu.so`` through its C ABI (``include/igapgpu.h``).
Arrays may be numpy arrays (host) or CUDA tensors (anything exposing
``data_ptr()``); the library detects device pointers itself.  There is no CPU
fallback: constructing an :class:`Assembly` without the built library or
without a GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libigapgpu.so")

LAW_GRADELAST, LAW_GRADELASTTIME, LAW_LINGRAD = 0, 1, 2
PREC_FP64, PREC_SPLIT, PREC_OZAKI = 0, 1, 2
REASON_REJECTED = -9  # igapgpu_solve: initial |F| above snes_f0_max
LAW_TORDER = {LAW_GRADELAST: 0, LAW_GRADELASTTIME: 2, LAW_LINGRAD: 0}
# default parameters of the reference plugins (phys/physgradelast.c:21,
# phys/physgradelasttime.c:21) and of the linear law
LAW_DEFAULT_PAR = {
    LAW_GRADELAST: [0.25, 0.50, 360., 180., 0.05, 1.0, 1.0, 1.e-3 * 0.5, 0.0],
    LAW_GRADELASTTIME: [0.25, 0.50, 500., 250., 0.025, 1.0, 1.0, 1.e-3 * 0.5, 0.0],
    LAW_LINGRAD: [1.0, 1.0, 0.1, 0, 0, 0, 0, 0, 0],
}


class IgapGpuError(RuntimeError):
    pass


class MeshDesc(ctypes.Structure):
    _fields_ = [("porder", ctypes.c_int), ("nelem", ctypes.c_int * 3),
                ("knots", ctypes.POINTER(ctypes.c_double) * 3),
                ("w", ctypes.POINTER(ctypes.c_double)), ("X", ctypes.POINTER(ctypes.c_double))]


class PhysDesc(ctypes.Structure):
    _fields_ = [("law", ctypes.c_int), ("par", ctypes.c_double * 9)]


class BCDesc(ctypes.Structure):
    _fields_ = [("bc_type", ctypes.c_int * 36), ("par_periodic", ctypes.c_double * 9),
                ("par_dirichlet", ctypes.c_double * 9), ("neumann", ctypes.c_double * 36)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("snes_abstol", ctypes.c_double), ("snes_rtol", ctypes.c_double),
                ("snes_stol", ctypes.c_double), ("snes_max_it", ctypes.c_int),
                ("linesearch", ctypes.c_int), ("ksp_restart", ctypes.c_int),
                ("ksp_rtol", ctypes.c_double), ("ksp_abstol", ctypes.c_double),
                ("ksp_dtol", ctypes.c_double), ("ksp_max_it", ctypes.c_int), ("pc", ctypes.c_int),
                ("use_graphs", ctypes.c_int), ("orth", ctypes.c_int), ("snes_f0_max", ctypes.c_double)]


class SolveStats(ctypes.Structure):
    _fields_ = [("newton_its", ctypes.c_int), ("ksp_its_total", ctypes.c_int),
                ("ksp_its_last", ctypes.c_int), ("converged", ctypes.c_int),
                ("reason", ctypes.c_int), ("fnorm0", ctypes.c_double), ("fnorm", ctypes.c_double)]


_lib = None


def lib():
    """Load libigapgpu.so (build it with ``python -m igap4_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise IgapGpuError(f"{LIBPATH} is missing: the CUDA extension must be built "
                               "(python -m igap4_gb300.build); there is no CPU fallback")
        L = ctypes.CDLL(LIBPATH)
        vp = ctypes.c_void_p
        L.igapgpu_assm_init.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(MeshDesc),
                                        ctypes.POINTER(PhysDesc), ctypes.POINTER(BCDesc), ctypes.c_int]
        L.igapgpu_finalize.argtypes = [vp]
        L.igapgpu_sizes.argtypes = [vp] + [ctypes.c_void_p] * 4
        L.igapgpu_pattern.argtypes = [vp, vp, vp]
        L.igapgpu_dirichlet.argtypes = [vp, vp, vp, vp]
        L.igapgpu_density.argtypes = [vp, vp, vp]
        L.igapgpu_sample_field.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
        L.igapgpu_debug_slot_counts.argtypes = [vp, vp]
        L.igapgpu_save_solution.argtypes = [vp, ctypes.c_char_p]
        L.igapgpu_load_solution.argtypes = [vp, ctypes.c_char_p]
        L.igapgpu_impose_dirichlet.argtypes = [vp, vp]
        for f in ("igapgpu_set_history", "igapgpu_get_history"):
            getattr(L, f).argtypes = [vp, ctypes.c_int, vp]
        L.igapgpu_shift_history.argtypes = [vp]
        for f in ("igapgpu_residual", "igapgpu_tangent", "igapgpu_matmult", "igapgpu_get_diagonal"):
            getattr(L, f).argtypes = [vp, vp, vp]
        L.igapgpu_get_diagonal.argtypes = [vp, vp]
        L.igapgpu_norm2.argtypes = [vp, vp, vp]
        L.igapgpu_assemble.argtypes = [vp, vp, vp, vp]
        L.igapgpu_ksp_solve.argtypes = [vp, vp, vp, ctypes.POINTER(SolverOpts),
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
        L.igapgpu_solve.argtypes = [vp, vp, ctypes.POINTER(SolverOpts), ctypes.POINTER(SolveStats)]
        L.igapgpu_default_solver_opts.argtypes = [ctypes.POINTER(SolverOpts)]
        L.igapgpu_default_solver_opts.restype = None
        L.igapgpu_set_precision.argtypes = [vp, ctypes.c_int]
        L.igapgpu_set_neumann.argtypes = [vp, vp]
        L.igapgpu_set_stream.argtypes = [vp, vp]
        L.igapgpu_synchronize.argtypes = [vp]
        L.igapgpu_last_error.restype = ctypes.c_char_p
        L.igapgpu_launch_count.restype = ctypes.c_int64
        L.igapgpu_profile.argtypes = [vp, ctypes.c_int]
        L.igapgpu_profile_read.argtypes = [vp, vp, vp, vp]
        L.igapgpu_profile_read_kind.argtypes = [vp, ctypes.c_int, vp, vp, vp]
        L.igapgpu_measure_fp64_peak.argtypes = [vp]
        L.igapgpu_measure_fp32_peak.argtypes = [vp]
        L.igapgpu_tc_selftest.argtypes = [ctypes.c_int, vp]
        L.igapgpu_wait_selftest.argtypes = [ctypes.c_int, ctypes.c_uint, vp]
        L.igapgpu_batch_init.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(MeshDesc),
                                         ctypes.POINTER(PhysDesc), ctypes.POINTER(BCDesc), ctypes.c_int]
        L.igapgpu_batch_info.argtypes = [vp, vp, vp, vp]
        L.igapgpu_batch_norms.argtypes = [vp, vp, vp]
        L.igapgpu_batch_set_schedule.argtypes = [vp, vp]
        L.igapgpu_batch_get_schedule.argtypes = [vp, vp]
        L.igapgpu_batch_autotune.argtypes = [vp, ctypes.c_int, ctypes.c_double, vp, vp, vp]
        _lib = L
    return _lib


CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


def _check(rc):
    if rc != 0:
        raise IgapGpuError(f"igapgpu error {rc}: {lib().igapgpu_last_error().decode()}")


def _ptr(a):
    """Raw pointer of a numpy array or a CUDA tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise IgapGpuError("tensor must be contiguous")
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise IgapGpuError("array must be C-contiguous")
    return ctypes.c_void_p(a.ctypes.data)


def beam_mesh(nelem, L=(1.0, 1.0, 1.0), porder=2, perturb=False):
    """Knot vectors, weights and control points of a box beam with a
    per-direction element count (the formulas of mesh/igabeam.c:34-72 and, with
    perturb, mesh/igabeamtest.c:68-70)."""
    knots = []
    for d in range(3):
        n = nelem[d]
        kv = np.empty(n + 1 + 2 * porder)
        l = 1.0 / n
        for k in range(len(kv)):
            kv[k] = 0.0 if k <= porder else ((k - porder) * l if k < n + porder else 1.0)
        knots.append(kv)
    nb = [n + porder for n in nelem]
    i, j, k = np.meshgrid(np.arange(nb[0]), np.arange(nb[1]), np.arange(nb[2]), indexing="ij")
    X = np.empty(nb + [3])
    X[..., 0] = (i - 0.5) / (nb[0] - 2) * L[0]
    X[..., 1] = (j - 0.5) / (nb[1] - 2) * L[1]
    X[..., 2] = (k - 0.5) / (nb[2] - 2) * L[2]
    if perturb:
        inside = ((i > 2) & (j > 2) & (k > 2) & (i < nb[0] - 2) & (j < nb[1] - 2) & (k < nb[2] - 2)).astype(float)
        ijk = i * k * j
        X[..., 0] += 0.2 * L[0] / nb[0] * inside * np.sin(3 * ijk)
        X[..., 1] += 0.2 * L[1] / nb[1] * inside * np.sin(5 * ijk)
        X[..., 2] += 0.2 * L[2] / nb[2] * inside * np.sin(7 * ijk)
    w = np.ones(nb[0] * nb[1] * nb[2])
    return knots, w, np.ascontiguousarray(X.reshape(-1))


def clamp_bc(faces=(0,), traction_face=None, traction=(0.0, 0.0, 0.0)):
    """bc_type / traction tables: listed faces clamped (both orders), others
    traction-free; optional constant traction on one face."""
    bct = np.ones(36, np.int32)
    neu = np.zeros(36)
    for f in faces:
        bct[6 * f:6 * f + 6] = 0
    if traction_face is not None:
        for d in range(3):
            neu[6 * traction_face + d] = traction[d]
    return bct, neu


def _descs(keep, nelem, knots, w, X, law, par, bc_type, neumann, par_dirichlet, porder=2):
    """ctypes descriptors of one instance; the arrays they point to go to keep."""
    arrs = [np.ascontiguousarray(k, np.float64) for k in knots]
    arrs += [np.ascontiguousarray(w, np.float64), np.ascontiguousarray(X, np.float64)]
    keep += arrs
    dp = ctypes.POINTER(ctypes.c_double)
    md = MeshDesc()
    md.porder = porder
    for d in range(3):
        md.nelem[d] = int(nelem[d])
        md.knots[d] = arrs[d].ctypes.data_as(dp)
    md.w = arrs[3].ctypes.data_as(dp)
    md.X = arrs[4].ctypes.data_as(dp)
    pd = PhysDesc()
    pd.law = law
    p = LAW_DEFAULT_PAR.get(law, [0.0] * 9) if par is None else list(par)
    for i in range(9):
        pd.par[i] = float(p[i]) if i < len(p) else 0.0
    bd = BCDesc()
    for i in range(36):
        bd.bc_type[i] = 1 if bc_type is None else int(bc_type[i])
        bd.neumann[i] = 0.0 if neumann is None else float(neumann[i])
    for i in range(9):
        bd.par_dirichlet[i] = 0.0 if par_dirichlet is None else float(par_dirichlet[i])
    return md, pd, bd


class Assembly:
    """One GPU assembly context (IGAPAssmInit + the Residual/Tangent callbacks)."""

    def __init__(self, nelem, knots, w, X, law=LAW_GRADELAST, par=None, bc_type=None,
                 neumann=None, par_dirichlet=None, nquad=4, porder=2):
        L = lib()
        self._keep = []
        md, pd, bd = _descs(self._keep, nelem, knots, w, X, law, par, bc_type, neumann, par_dirichlet, porder)
        h = ctypes.c_void_p()
        _check(L.igapgpu_assm_init(ctypes.byref(h), ctypes.byref(md), ctypes.byref(pd),
                                   ctypes.byref(bd), nquad))
        self.h = h
        self._sizes()
        self.nelem = tuple(int(n) for n in nelem)

    def _sizes(self):
        nd, nz, el = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        to = ctypes.c_int()
        _check(lib().igapgpu_sizes(self.h, ctypes.byref(nd), ctypes.byref(nz), ctypes.byref(to),
                                   ctypes.byref(el)))
        self.ndof, self.nnz, self.torder, self.nelem_total = nd.value, nz.value, to.value, el.value

    def close(self):
        if getattr(self, "h", None):
            lib().igapgpu_finalize(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pattern(self):
        rowptr = np.zeros(self.ndof + 1, np.int64)
        cols = np.zeros(self.nnz, np.int32)
        _check(lib().igapgpu_pattern(self.h, _ptr(rowptr), _ptr(cols)))
        return rowptr, cols

    def dirichlet(self):
        """(rows int64, prescribed values float64) of the Dirichlet DOFs."""
        n = ctypes.c_int64()
        _check(lib().igapgpu_dirichlet(self.h, ctypes.byref(n), None, None))
        rows = np.zeros(n.value, np.int64)
        vals = np.zeros(n.value)
        if n.value:
            _check(lib().igapgpu_dirichlet(self.h, ctypes.byref(n), _ptr(rows), _ptr(vals)))
        return rows, vals

    def density(self):
        """Densities of the law integrated over the body on the current state
        (iga_intdensity of the reference)."""
        HH = np.zeros(16)
        n = ctypes.c_int()
        _check(lib().igapgpu_density(self.h, _ptr(HH), ctypes.byref(n)))
        return HH[:n.value].copy()

    def sample_field(self, nppe):
        """The law's field on the plot lattice of iga_plotfield (nppe samples
        per element and direction plus the far faces) at the current state:
        field [NX, NY, NZ, nfield], knot coordinates xq and positions X
        [NX, NY, NZ, 3], NX = nppe * nelem[0] + 1."""
        nf = ctypes.c_int()
        npts = ctypes.c_int64()
        _check(lib().igapgpu_sample_field(self.h, int(nppe), None, None, None, ctypes.byref(nf), ctypes.byref(npts)))
        shape = tuple(int(nppe) * int(n) + 1 for n in self.nelem)
        F = np.zeros(shape + (nf.value,))
        xq = np.zeros(shape + (3,))
        X = np.zeros(shape + (3,))
        _check(lib().igapgpu_sample_field(self.h, int(nppe), _ptr(F), _ptr(xq), _ptr(X), None, None))
        return F, xq, X

    def debug_slot_counts(self):
        """Per CSR slot, the element contributions a plain read-modify-write
        scatter (colour by colour) lands in it: the race check of the colouring."""
        out = np.zeros(self.nnz)
        _check(lib().igapgpu_debug_slot_counts(self.h, _ptr(out)))
        return out

    def save_solution(self, fname):
        """Write the reference's solution file (IGAPSolvSaveSolution layout)."""
        _check(lib().igapgpu_save_solution(self.h, os.fsencode(fname)))

    def load_solution(self, fname):
        """Read a solution file written by the reference or by save_solution."""
        _check(lib().igapgpu_load_solution(self.h, os.fsencode(fname)))

    def impose_dirichlet(self, U):
        """U[r] = g_r on the Dirichlet rows, in place (host array or CUDA tensor)."""
        _check(lib().igapgpu_impose_dirichlet(self.h, _ptr(U)))
        return U

    def set_history(self, level, U):
        _check(lib().igapgpu_set_history(self.h, level, _ptr(U)))

    def get_history(self, level, out=None):
        out = np.zeros(self.ndof) if out is None else out
        _check(lib().igapgpu_get_history(self.h, level, _ptr(out)))
        return out

    def shift_history(self):
        _check(lib().igapgpu_shift_history(self.h))

    def set_state(self, U_hist):
        """U_hist: (torder+1, ndof) array; row 0 is the current iterate."""
        for lvl in range(self.torder + 1):
            self.set_history(lvl, np.ascontiguousarray(U_hist[lvl]) if isinstance(U_hist, np.ndarray) else U_hist[lvl])

    def residual(self, U=None, out=None):
        out = np.zeros(self.ndof) if out is None else out
        _check(lib().igapgpu_residual(self.h, _ptr(U), _ptr(out)))
        return out

    def tangent(self, U=None, out=None):
        out = np.zeros(self.nnz) if out is None else out
        _check(lib().igapgpu_tangent(self.h, _ptr(U), _ptr(out)))
        return out

    def assemble(self, U=None, RR=None, vals=None):
        _check(lib().igapgpu_assemble(self.h, _ptr(U), _ptr(RR), _ptr(vals)))
        return RR, vals

    def tangent_internal(self, U=None):
        """Assemble into the context's own matrix (used by matmult / solve)."""
        _check(lib().igapgpu_tangent(self.h, _ptr(U), None))

    def matmult(self, x, y=None):
        y = np.zeros(self.ndof) if y is None else y
        _check(lib().igapgpu_matmult(self.h, _ptr(x), _ptr(y)))
        return y

    def norm2(self, x):
        """FP64 2-norm of a context-sized vector (host array or CUDA tensor)."""
        out = ctypes.c_double()
        _check(lib().igapgpu_norm2(self.h, _ptr(x), ctypes.byref(out)))
        return out.value

    def diagonal(self, out=None):
        out = np.zeros(self.ndof) if out is None else out
        _check(lib().igapgpu_get_diagonal(self.h, _ptr(out)))
        return out

    @staticmethod
    def default_opts(**kw):
        o = SolverOpts()
        lib().igapgpu_default_solver_opts(ctypes.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def ksp_solve(self, b, x, **kw):
        o = self.default_opts(**kw)
        its = ctypes.c_int()
        rn = ctypes.c_double()
        _check(lib().igapgpu_ksp_solve(self.h, _ptr(b), _ptr(x), ctypes.byref(o), ctypes.byref(its),
                                       ctypes.byref(rn)))
        return its.value, rn.value

    def solve(self, U, **kw):
        o = self.default_opts(**kw)
        st = SolveStats()
        _check(lib().igapgpu_solve(self.h, _ptr(U), ctypes.byref(o), ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in SolveStats._fields_}

    def set_neumann(self, table):
        """New constant traction table (36 entries); recomputes the Neumann load."""
        t = np.ascontiguousarray(table, np.float64)
        _check(lib().igapgpu_set_neumann(self.h, _ptr(t)))

    def set_precision(self, mode):
        _check(lib().igapgpu_set_precision(self.h, mode))

    def set_stream(self, stream_handle):
        """stream_handle: an integer cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream),
        or None for the context's own stream.  0 is the legacy default stream
        (torch's default stream) and is passed as cudaStreamLegacy, because a
        NULL handle selects the context's own stream."""
        if stream_handle is None:
            h = None
        else:
            h = ctypes.c_void_p(int(stream_handle) or CUDA_STREAM_LEGACY)
        _check(lib().igapgpu_set_stream(self.h, h))

    def synchronize(self):
        _check(lib().igapgpu_synchronize(self.h))

    def profile(self, enable=True):
        _check(lib().igapgpu_profile(self.h, int(enable)))

    def profile_read(self, kind=-1):
        """(ms, launches, elements) of the timed element kernels; kind 0 = the
        residual / FP64 element kernel, 1 = tensor-core tangent kernel, 2 = the
        nonlinear laws' all-points law kernel, -1 = all."""
        ms = ctypes.c_double()
        nl, ne = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().igapgpu_profile_read_kind(self.h, kind, ctypes.byref(ms), ctypes.byref(nl),
                                               ctypes.byref(ne)))
        return ms.value, nl.value, ne.value


def launch_count() -> int:
    return int(lib().igapgpu_launch_count())


def tc_selftest(variant=0):
    """Run the tcgen05 self-test GEMM; returns (D, expected) as (128, 32) arrays."""
    out = np.zeros(128 * 32, np.float32)
    _check(lib().igapgpu_tc_selftest(variant, _ptr(out)))
    r = np.arange(128)[:, None]
    n = np.arange(32)[:, None]
    k = np.arange(16)[None, :]
    A = ((r * 3 + k * 5) % 7) - 3
    B = ((n * 2 + k * 3) % 5) - 2
    return out.reshape(128, 32), (A @ B.T).astype(np.float32)


def measure_fp64_peak() -> float:
    t = ctypes.c_double()
    _check(lib().igapgpu_measure_fp64_peak(ctypes.byref(t)))
    return t.value


def measure_fp32_peak() -> float:
    t = ctypes.c_double()
    _check(lib().igapgpu_measure_fp32_peak(ctypes.byref(t)))
    return t.value


class BatchSchedule(ctypes.Structure):
    """Work-queue schedule of the batched kernels (igapgpu_batch_schedule)."""
    _fields_ = [("grab_fp64", ctypes.c_int), ("ctas_per_sm_fp64", ctypes.c_int),
                ("grab_tc", ctypes.c_int), ("order", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchAssembly(Assembly):
    """Independent instances (beams of different sizes and parameters, one law)
    assembled by one persistent launch per kernel.  The object behaves as an
    :class:`Assembly` of the block-diagonal union: DOFs of instance i occupy
    ``dof_off[i]:dof_off[i+1]``.

    instances: sequence of dicts with keys nelem, knots, w, X and optionally
    par, bc_type, neumann, par_dirichlet."""

    def __init__(self, instances, law=LAW_LINGRAD, nquad=4):
        L = lib()
        n = len(instances)
        self._keep = []
        mds, pds, bds = (MeshDesc * n)(), (PhysDesc * n)(), (BCDesc * n)()
        for i, inst in enumerate(instances):
            md, pd, bd = _descs(self._keep, inst["nelem"], inst["knots"], inst["w"], inst["X"], law,
                                inst.get("par"), inst.get("bc_type"), inst.get("neumann"),
                                inst.get("par_dirichlet"))
            mds[i], pds[i], bds[i] = md, pd, bd
        h = ctypes.c_void_p()
        _check(L.igapgpu_batch_init(ctypes.byref(h), n, mds, pds, bds, nquad))
        self.h = h
        self._sizes()
        self.ninst = n
        self.dof_off = np.zeros(n + 1, np.int64)
        self.elem_off = np.zeros(n + 1, np.int64)
        ni = ctypes.c_int()
        _check(L.igapgpu_batch_info(h, ctypes.byref(ni), _ptr(self.dof_off), _ptr(self.elem_off)))
        self.nelem = None
        self.instance_nelem = [tuple(int(v) for v in inst["nelem"]) for inst in instances]

    def norms(self, x):
        """FP64 2-norm of every instance's segment of x (host array or CUDA tensor)."""
        out = np.zeros(self.ninst)
        _check(lib().igapgpu_batch_norms(self.h, _ptr(x), _ptr(out)))
        return out

    def segment(self, x, i):
        return x[self.dof_off[i]:self.dof_off[i + 1]]

    @property
    def schedule(self):
        s = BatchSchedule()
        _check(lib().igapgpu_batch_get_schedule(self.h, ctypes.byref(s)))
        return s.as_dict()

    @schedule.setter
    def schedule(self, d):
        s = BatchSchedule(**{k: int(v) for k, v in d.items()})
        _check(lib().igapgpu_batch_set_schedule(self.h, ctypes.byref(s)))

    def autotune(self, reps=2, frac=0.1):
        """Time the candidate schedules, keep the fastest; returns
        (schedule dict, best FP64-kernel ms, best tensor-core-kernel ms) on
        the timed queue prefix."""
        s = BatchSchedule()
        m64, mtc = ctypes.c_double(), ctypes.c_double()
        _check(lib().igapgpu_batch_autotune(self.h, int(reps), float(frac), ctypes.byref(s),
                                            ctypes.byref(m64), ctypes.byref(mtc)))
        return s.as_dict(), m64.value, mtc.value


def batch_instances(n=256, seed=0, nx=(8, 64), nyz=(2, 16), lam=(0.5, 2.0), mu=(0.5, 2.0),
                    ell=(0.02, 0.2), L=(4.0, 1.0, 1.0), traction=1e-3, clamp=True):
    """Seeded uneven beam instances of the linear strain-gradient law: nx
    uniform in nx[0]..nx[1], ny = nz uniform in nyz[0]..nyz[1], lambda, mu,
    length scale uniform in their ranges; clamped at x = 0, uniform traction
    in -z at x = L (the 16x4x4 beam problem's boundary conditions)."""
    rng = np.random.default_rng(seed)
    out = []
    bct, neu = clamp_bc((0,) if clamp else (), traction_face=1, traction=(0.0, 0.0, -traction))
    for _ in range(n):
        ex = int(rng.integers(nx[0], nx[1] + 1))
        eyz = int(rng.integers(nyz[0], nyz[1] + 1))
        nelem = (ex, eyz, eyz)
        knots, w, X = beam_mesh(nelem, L)
        par = [rng.uniform(*lam), rng.uniform(*mu), rng.uniform(*ell), 0, 0, 0, 0, 0, 0]
        out.append(dict(nelem=nelem, knots=knots, w=w, X=X, par=par, bc_type=bct, neumann=neu))
    return out


def wait_selftest(target, limit=1 << 16):
    """Bounded device wait on a counter that nothing increments (target 1) or
    that is already reached (target 0); returns the device error word."""
    st = ctypes.c_int(-1)
    _check(lib().igapgpu_wait_selftest(int(target), int(limit), ctypes.byref(st)))
    return st.value

"""Time stepping of the three-level transient law on the device.

The reference library has no time loop: its callers set the history levels
U_hist[1] = u_n, U_hist[2] = u_{n-1} (include/coreimpl.h:17,
phys/gradelasttime.c:9-11), call IGAPSolvSolve and shift the levels.  This
module is that caller for the transient runs: a seeded tip traction
(sum of sinusoids), one Newton solve per step with u_n as the initial
iterate (or a predictor's guess), then the history shift.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

REASON_REJECTED = -9  # igapgpu_solve: initial |F| above snes_f0_max


@dataclass
class TipLoad:
    """Traction on one face: sum_i a_i sin(2 pi f_i t) along one direction,
    amplitudes uniform in [0, amax], frequencies uniform in [fmin, fmax]."""

    seed: int
    n: int = 4
    amax: float = 1e-3
    fmin: float = 0.5
    fmax: float = 5.0
    face: int = 1        # x = L (the tip of the beam)
    dof: int = 2         # z component
    sign: float = -1.0
    amp: np.ndarray = field(init=False)
    freq: np.ndarray = field(init=False)

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        self.amp = rng.uniform(0.0, self.amax, self.n)
        self.freq = rng.uniform(self.fmin, self.fmax, self.n)

    def value(self, t: float) -> float:
        return self.sign * float(np.sum(self.amp * np.sin(2.0 * np.pi * self.freq * t)))

    def table(self, t: float) -> np.ndarray:
        tab = np.zeros(36)
        tab[6 * self.face + self.dof] = self.value(t)  # order 0 (plain traction)
        return tab


@dataclass
class StepRecord:
    t: float
    newton_its: int
    ksp_its: int
    fnorm0: float
    fnorm: float
    converged: int
    seconds: float
    used_prediction: bool = False


def run_transient(A, load: TipLoad, nsteps: int, dt: float, predictor=None, opts=None,
                  record_states: bool = True, device=None, log=None, start=None):
    """Advance `nsteps` steps of size dt (dt must equal the law's par[7]).

    A: igap4_gb300.Assembly with the transient law.  predictor: optional
    callable (u_n, u_nm1, dload) -> guess for u_{n+1}, or an object whose
    candidates(u_n, u_nm1, dload) lists guesses; a guess is kept only if it
    lowers the residual norm below that of u_n (plain Newton fallback).
    log: optional callable, given each StepRecord as it is made.
    start: optional (u_n, u_{n-1}, n0): continue a trajectory after step n0
    (device FP64 vectors) instead of starting from rest.
    Returns (states [nsteps+1, ndof] or None, list of StepRecord); the
    state where the run ended is left in run_transient.last as
    (u_n, u_{n-1}, n), a `start` for the next run."""
    import torch

    dev = device or torch.device("cuda")
    # the context works on torch's current stream, so residuals read by torch
    # (the predictor's acceptance test) are ordered after the kernels
    A.set_stream(torch.cuda.current_stream(dev).cuda_stream)
    o = dict(snes_abstol=1e-8, ksp_rtol=1e-5, ksp_restart=100, ksp_max_it=5000, snes_max_it=30, use_graphs=1)
    if opts:
        o.update(opts)
    zero = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    n0 = 0
    u_n = zero.clone()
    u_nm1 = zero.clone()
    if start is not None:
        u_n, u_nm1, n0 = start[0].clone(), start[1].clone(), int(start[2])
    A.set_history(1, u_n)
    A.set_history(2, u_nm1)
    states = [u_n.cpu().numpy()] if record_states else None
    recs = []
    F = torch.zeros_like(zero)
    prev_load = load.value(n0 * dt) if n0 > 0 else 0.0
    for n in range(n0, n0 + nsteps):
        t = (n + 1) * dt
        A.set_neumann(load.table(t))
        t0 = time.perf_counter()
        U = u_n.clone()
        used = False
        st = None
        if predictor is not None:
            # the Newton correction leaves Dirichlet DOFs where the initial
            # iterate puts them (their columns are cleared), so every guess
            # carries the prescribed values exactly
            dl = load.value(t) - prev_load
            cands = predictor.candidates(u_n, u_nm1, dl) if hasattr(predictor, "candidates") \
                else [predictor(u_n, u_nm1, dl)]
            A.residual(U, F)
            f_plain = A.norm2(F)
            if len(cands) == 1:
                # Newton from the guess, unless its residual is above that of
                # u_n (the solve then stops before its first step and the
                # step falls back to plain Newton from u_n)
                guess = A.impose_dirichlet(cands[0].contiguous())
                st = A.solve(guess, **dict(o, snes_f0_max=f_plain))
                if st["reason"] == REASON_REJECTED:
                    st = None
                else:
                    U, used = guess, True
            else:  # several guesses: the one with the smallest residual
                best = f_plain
                for g in cands:
                    guess = A.impose_dirichlet(g.contiguous())
                    A.residual(guess, F)
                    f_pred = A.norm2(F)
                    if f_pred < best:
                        best = f_pred
                        U = guess.clone()
                        used = True
        if st is None:
            st = A.solve(U, **o)
        A.synchronize()
        dtm = time.perf_counter() - t0
        recs.append(StepRecord(t, st["newton_its"], st["ksp_its_total"], st["fnorm0"], st["fnorm"],
                               st["converged"], dtm, used))
        if log:
            log(recs[-1])
        # history shift: u_{n-1} <- u_n, u_n <- u_{n+1}
        A.set_history(0, U)
        A.shift_history()
        u_nm1, u_n = u_n, U
        prev_load = load.value(t)
        if record_states:
            states.append(U.cpu().numpy())
    run_transient.last = (u_n, u_nm1, n0 + nsteps)
    return (np.array(states) if record_states else None), recs


def step_breakdown(A, load, dt, opts, reps=5):
    """Where one transient step's time goes, after a run_transient call (its
    last state u_n, the history it left): the residual and the tangent assembly
    alone (synchronised wall clock; the law kernel, the residual/FP64 element kernel and
    the tensor-core tangent kernel from the library's profiling), then one
    step's Newton solve from u_n (Newton and GMRES iterations, wall ms), and
    the ms per GMRES iteration once the assemblies are taken out."""
    import torch

    dev = torch.device("cuda")
    u_n, _, n = run_transient.last
    U = u_n.clone().to(dev)
    RR = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    K = torch.zeros(A.nnz, dtype=torch.float64, device=dev)
    out = {}
    for name, fn in (("residual", lambda: A.residual(U, RR)), ("tangent", lambda: A.tangent(U, K))):
        fn()
        A.synchronize()
        A.profile(True)
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        A.synchronize()
        host_ms = 1e3 * (time.perf_counter() - t0) / reps
        kinds = {k: A.profile_read(k)[0] / reps for k in (2, 0, 1)}
        A.profile(False)
        out[name] = {"ms": host_ms, "law_kernel_ms": kinds[2],
                     "residual_or_fp64_kernel_ms": kinds[0], "tensor_core_kernel_ms": kinds[1]}
    # the next step's solve from u_n
    A.set_neumann(load.table((n + 1) * dt))
    guess = u_n.clone().to(dev)
    A.synchronize()
    t0 = time.perf_counter()
    st = A.solve(guess, **opts)
    A.synchronize()
    solve_ms = 1e3 * (time.perf_counter() - t0)
    its, kits = st["newton_its"], st["ksp_its_total"]
    # a Newton solve of `its` iterations assembles its + 1 residuals and its tangents
    assembly_ms = (its + 1) * out["residual"]["ms"] + its * out["tangent"]["ms"]
    out["solve"] = {"ms": solve_ms, "newton_its": its, "gmres_its": kits, "converged": st["converged"],
                    "ms_per_gmres_its_excluding_assembly": (solve_ms - assembly_ms) / max(kits, 1),
                    "note": "assembly time taken as (its + 1) residuals and its tangents"}
    return out


def main():
    """Config-3 style run: the transient beam under a seeded tip-load history,
    plain Newton from u_n (or a saved predictor), per-step records as JSON.

        python -m igap4_gb300.transient --nelem 64,16,16 --steps 400 --seed 0 --prec split
    """
    import argparse
    import json

    import numpy as np  # noqa: F811

    ap = argparse.ArgumentParser()
    ap.add_argument("--nelem", default="64,16,16")
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--dt", type=float, default=1e-2)
    ap.add_argument("--amax", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--prec", default="split", choices=["fp64", "split"])
    ap.add_argument("--pc", type=int, default=3,
                    help="GMRES preconditioner: 1 Jacobi, 2 point blocks, 3 cell blocks (default: 72 "
                         "against 166 Jacobi iterations per step at 64x16x16), 4 additive Schwarz")
    ap.add_argument("--predictor", default=None, help=".npz written by train_predictor --save")
    ap.add_argument("--states", default=None, help="write the trajectory (FP64 states) to this .npy")
    ap.add_argument("--orth", type=int, default=1, help="GMRES orthogonalisation: 0 MGS, 1 CGS2")
    ap.add_argument("--breakdown", action="store_true",
                    help="after the run, time one step's parts on the last state (assembly kernels, "
                         "Newton and GMRES iterations, ms per GMRES iteration)")
    a = ap.parse_args()
    import sys
    import torch  # noqa: F401

    from .train_predictor import load_network, transient_problem

    nelem = tuple(int(v) for v in a.nelem.split(","))
    A, _ = transient_problem(nelem, a.dt, prec=a.prec)
    pred = None
    if a.predictor:
        from .predictor import LearnedPredictor

        net, sc = load_network(a.predictor, tuple(n + 2 for n in nelem))
        pred = LearnedPredictor(net, sc, A=A)
    load = TipLoad(seed=a.seed, amax=a.amax)
    opts = dict(snes_abstol=1e-8, ksp_rtol=1e-5, ksp_restart=100, ksp_max_it=5000, snes_max_it=30,
                use_graphs=1, pc=a.pc, orth=a.orth)

    def log(r):  # one line per step on stderr, as it happens
        print(f"t {r.t:.4f} newton {r.newton_its} ksp {r.ksp_its} |F| {r.fnorm0:.3e} -> {r.fnorm:.3e} "
              f"conv {r.converged} {1e3 * r.seconds:.1f} ms pred {int(r.used_prediction)}", file=sys.stderr,
              flush=True)

    t0 = time.perf_counter()
    states, recs = run_transient(A, load, a.steps, a.dt, predictor=pred, opts=opts,
                                 record_states=a.states is not None, log=log)
    wall = time.perf_counter() - t0
    if a.states:
        np.save(a.states, states)
    its = np.array([r.newton_its for r in recs])
    kits = np.array([r.ksp_its for r in recs])
    ms = np.array([1e3 * r.seconds for r in recs])
    out = {"nelem": list(nelem), "ndof": A.ndof, "steps": a.steps, "dt": a.dt, "seed": a.seed,
           "load": {"amp": load.amp.tolist(), "freq": load.freq.tolist()}, "prec": a.prec, "pc": a.pc,
           "predictor": a.predictor, "wall_s": wall, "converged_all": bool(all(r.converged for r in recs)),
           "newton_its_per_step": float(its.mean()), "ksp_its_per_step": float(kits.mean()),
           "ms_per_step": float(ms.mean()), "max_fnorm": float(max(r.fnorm for r in recs)),
           "records": [{"t": r.t, "newton": r.newton_its, "ksp": r.ksp_its, "f0": r.fnorm0, "f": r.fnorm,
                        "ms": 1e3 * r.seconds, "pred": r.used_prediction} for r in recs]}
    if a.breakdown:
        out["breakdown"] = step_breakdown(A, load, a.dt, opts)
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""Run one assembly configuration on the GPU a fixed number of times (for
profilers and quick timings).

    python -m igap4_gb300.run_case --nelem 64,16,16 --prec fp64 --what assemble --reps 2

--what: assemble (residual + tangent), residual, tangent, spmv (after one
assembly), batch (seeded uneven instances, --ninst of them), solve (Newton-
GMRES from U = 0 with preconditioner --pc: 0 none, 1 Jacobi, 2 point-block
Jacobi, 3 cell-block Jacobi, 4 additive Schwarz; prints Newton and Krylov
iterations).  --prec fp64 | split | fp64q (the FP64-quality tensor-core
tangent), --porder 2 | 3.  Prints the wall time of each repetition after the
first.
"""
from __future__ import annotations

import argparse
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nelem", default="64,16,16")
    ap.add_argument("--prec", default="fp64", choices=["fp64", "split", "fp64q"])
    ap.add_argument("--porder", type=int, default=2, choices=[2, 3])
    ap.add_argument("--what", default="assemble",
                    choices=["assemble", "residual", "tangent", "spmv", "batch", "solve"])
    ap.add_argument("--pc", type=int, default=1)
    ap.add_argument("--ksp-rtol", type=float, default=1e-6)
    ap.add_argument("--abstol", type=float, default=1e-10)
    ap.add_argument("--law", default="lingrad", choices=["lingrad", "gradelast", "gradelasttime"])
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--ninst", type=int, default=32)
    a = ap.parse_args()
    import torch

    import igap4_gb300 as ig

    law = {"lingrad": ig.LAW_LINGRAD, "gradelast": ig.LAW_GRADELAST, "gradelasttime": ig.LAW_GRADELASTTIME}[a.law]
    if a.what == "batch":
        insts = ig.batch_instances(a.ninst, seed=1, nx=(8, 32), nyz=(2, 8))
        A = ig.BatchAssembly(insts, law=ig.LAW_LINGRAD)
    else:
        nelem = tuple(int(v) for v in a.nelem.split(","))
        bct, neu = ig.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
        knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0), a.porder)
        par = (1.0, 1.0, 0.1) if law == ig.LAW_LINGRAD else None
        A = ig.Assembly(nelem, knots, w, X, law=law, par=par, bc_type=bct, neumann=neu, porder=a.porder)
    A.set_precision({"split": ig.PREC_SPLIT, "fp64q": ig.PREC_OZAKI}.get(a.prec, ig.PREC_FP64))
    dev = torch.device("cuda")
    U = torch.tensor(np.random.default_rng(1).uniform(-1e-2, 1e-2, A.ndof), device=dev)
    RR = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    x = torch.tensor(np.random.default_rng(2).standard_normal(A.ndof), device=dev)
    y = torch.zeros_like(x)
    if a.what == "spmv":
        A.assemble(U, RR, None)
    if a.what == "solve":
        for k in range(a.reps):
            Z = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
            A.synchronize()
            t0 = time.perf_counter()
            st = A.solve(Z, snes_abstol=a.abstol, ksp_rtol=a.ksp_rtol, ksp_restart=100, ksp_max_it=200000,
                         snes_max_it=20, pc=a.pc, use_graphs=1)
            A.synchronize()
            print(f"rep {k}: {1e3 * (time.perf_counter() - t0):.1f} ms, newton {st['newton_its']}, "
                  f"gmres {st['ksp_its_total']}, |F| {st['fnorm0']:.3e} -> {st['fnorm']:.3e}, "
                  f"converged {st['converged']}")
        print(f"elements {A.nelem_total} ndof {A.ndof} nnz {A.nnz} pc {a.pc}")
        return
    for k in range(a.reps):
        A.synchronize()
        t0 = time.perf_counter()
        if a.what in ("assemble", "batch"):
            A.assemble(U, RR, None)
        elif a.what == "residual":
            A.residual(U, RR)
        elif a.what == "tangent":
            A.tangent(U, None)
        else:
            A.matmult(x, y)
        A.synchronize()
        if k:
            print(f"rep {k}: {1e3 * (time.perf_counter() - t0):.3f} ms")
    print(f"elements {A.nelem_total} ndof {A.ndof} nnz {A.nnz}")


if __name__ == "__main__":
    main()

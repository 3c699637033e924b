"""Benchmark: residual + tangent assembly of the 128 x 32 x 32 quadratic beam.

One step = one fused assembly of the residual Vec and the CSR tangent of the
whole beam (131,072 elements, 64 Gauss points each) on the GPU, state already
resident in HBM.  Metric: assembled elements/s.  The headline is the
FP64-quality mode (residual in double-FP32 arithmetic on the FP32 pipe;
tangent on the tensor cores from error-free BF16 slices of the Gram operands;
both errors against the FP64 kernels measured in the same run); the pure FP64
and the TF32x3 split modes follow in `modes`.
Also reported:

* e2e  -- the same step through the C ABI with HOST buffers (state in from
  pinned host memory, residual back to pinned host memory; the tangent stays
  in the device matrix that MatMult uses), copies inside the timed region;
* roofline -- the dominant kernel of the headline mode against the measured
  peak of the pipe or memory that bounds it;
* spmv -- CSR SpMV (the MATSHELL multiply) GB/s over repeated multiplies;
* batched -- 256 seeded uneven beams in persistent launches;
* transient -- time to |F| <= 1e-8 per step of the transient law, plain
  Newton against the learned predictor;
* cpu_baseline -- the CPU oracle port (the reference's loop structure,
  restated in C) on the host cores, on a bounded element sample.

`--impl reference` times the CPU path alone (the reference's assembly
restated in C; the reference's sources are not available on the GPU host).
Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
launching stream; the L2 is flushed (256 MiB write) before every timed step.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NELEM = (128, 32, 32)
LBEAM = (4.0, 1.0, 1.0)
LAW_PAR = (1.0, 1.0, 0.1)  # lambda, mu, ell
SEED = 20261203
# algorithmic cost per element (p = 2, 64 points, 81 DOFs)
TAN_FLOP_PER_ELEM = 2 * 64 * (30 * 27 * 3 * 10 + 81 * 81 * 10)  # 11,508,480
RES_FLOP_PER_ELEM = 2 * 64 * (27 * 30 + 27 * 30)                 # 207,360
# FLOPs the kernels execute for the linear law (Gram form of the tangent):
# FP64 kernel: 378 basis pairs x 64 points x 72 (Gram sums) + 64 x 243
# (weighted derivatives) + 64 x 3,420 (state interpolation, law, projection)
# + block formation and scatter
EXEC_FLOP_FP64_ELEM = 378 * 64 * 72 + 64 * 243 + 64 * 3420 + 30_000  # ~2.0 M
# tensor-core kernel: 3 TF32 products of M128 x N96 x K256 per element
EXEC_FLOP_TC_ELEM = 3 * 2 * 128 * 96 * 256                         # 18.9 M
# FP64-quality tensor-core kernel: 12 BF16 products of M128 x N96 x K256 per element
EXEC_FLOP_OZ_ELEM = 12 * 2 * 128 * 96 * 256                        # 75.5 M
# residual-only FP64 kernel: state interpolation, law and projection per point
EXEC_FLOP_RES_ELEM = 64 * 3420 + 64 * 243
# double-FP32 residual kernel (res_df_kernel), FP32-pipe lane instructions per
# point: 2 x 729 compensated dot-product terms of 12 instructions
# (interpolation, projection), the law in pair arithmetic (~1,090), pair
# renormalisations (324) and the per-warp column sums (~863)
EXEC_F32_RES_DF_ELEM = 64 * (2 * 729 * 12 + 1090 + 324 + 863)
# its HBM bytes per element: the pair cache (64 points x 244 pairs) and the
# element's 81 residual pairs
ALG_BYTES_RES_DF_ELEM = 64 * 244 * 8 + 81 * 8
# FP64-quality tangent: per element the slices (8 chunks x 22,528 B), the row
# exponents (88 B) and the read-modify-write of its 6,561 FP64 CSR slots
ALG_BYTES_OZ_ELEM = 8 * 22528 + 88 + 2 * 8 * 6561
# cached-operand tensor-core tangent: per element the operands (8 chunks x
# 11,264 B) and the read-modify-write of its 6,561 FP64 CSR slots
ALG_BYTES_TCS_ELEM = 8 * 11264 + 2 * 8 * 6561
# Measured DRAM traffic per element (dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture of the kernel on a smaller mesh, divided by the elements
# the launch processed; the bench scales it by the elements per launch): FP64
# fused kernel (64x16x16, one colour launch of 792 elements: 218.6 MB), TF32x3
# tangent (64x16x16, 792 elements: 155.2 MB), FP64-quality tangent (48x16x16,
# 455 elements on 16 CTAs: 170.0 MB), double-FP32 residual (48x16x16, 12,288
# elements: 2.057 GB)
TRAFFIC_FP64_ELEM = 218.6e6 / 792
TRAFFIC_TCS_ELEM = 155.2e6 / 792
TRAFFIC_OZ_ELEM = 170.0e6 / 455
TRAFFIC_RES_DF_ELEM = 2.057e9 / 12288


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--nelem", default="128,32,32")
    ap.add_argument("--prec", default="all", choices=["fp64q", "fp64", "split", "all"],
                    help="all: the FP64-quality tensor-core mode as the headline, then the FP64 and the "
                         "split modes")
    ap.add_argument("--spmv", type=int, default=200, help="SpMV repetitions")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch", type=int, default=256,
                    help="instances of the batched workload (0 skips it)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--transient-steps", type=int, default=40,
                    help="time steps of the transient workload per arm (0 skips it)")
    ap.add_argument("--transient-nelem", default="64,16,16")
    ap.add_argument("--gradelast-nelem", default="64,16,16",
                    help="the reference's static law assembled at this size ('0' skips the block)")
    return ap.parse_args()


# ------------------------------------------------------------------ CPU
def _cpu_worker(args):
    """Time the oracle port on `nel` elements of a 32x8x8 beam (same element
    kind: p=2, 64 points, linear law); returns (elements, seconds)."""
    nel, seed = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    bct, neu = po.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    prob = po.Problem(nelem=(32, 8, 8), L=LBEAM, law=po.LAW_LINGRAD, par=np.array(LAW_PAR + (0,) * 6),
                      bc_type=bct, neumann=neu)
    case = po.OracleCase(prob)
    U = po.random_state(prob, seed)
    t0 = time.perf_counter()
    case.residual_elements(U, 0, nel)
    case.tangent_elements(U, 0, nel)
    return nel, time.perf_counter() - t0


def _cpu_worker_law(args):
    """Time the oracle port on `nel` elements of a 16x4x4 beam with the
    reference's static law (gradelast, its default material); returns
    (elements, seconds)."""
    nel, seed = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    prob = po.Problem(nelem=(16, 4, 4), law=po.LAW_GRADELAST)
    case = po.OracleCase(prob)
    U = po.random_state(prob, seed)
    t0 = time.perf_counter()
    case.residual_elements(U, 0, nel)
    case.tangent_elements(U, 0, nel)
    return nel, time.perf_counter() - t0


def cpu_rate(seconds: float, cores: int):
    """Aggregate elements/s of `cores` concurrent single-threaded processes."""
    # calibrate with a tiny sample on one core
    n1, t1 = _cpu_worker((8, SEED))
    per_el = t1 / n1
    nel = max(8, int(seconds / per_el))
    nel = min(nel, 32 * 8 * 8)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_worker, [(nel, SEED + i) for i in range(cores)])
        wall = time.perf_counter() - t0
    tot = sum(r[0] for r in res)
    slowest = max(r[1] for r in res)
    return tot / slowest, nel, slowest, wall


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    if not os.path.exists(po.LIBORC):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_oracle.sh")], check=True,
                       stdout=subprocess.DEVNULL)
    cores = os.cpu_count() or 1
    rates = []
    for _ in range(a.warmup):
        cpu_rate(2.0, cores)
    sample = None
    sample_s = []
    for _ in range(a.steps):
        r, nel, slowest, wall = cpu_rate(max(2.0, a.cpu_seconds / max(a.steps, 1)), cores)
        rates.append(r)
        sample_s.append(slowest)
        sample = f"{cores} processes x {nel} elements (p=2, 64 Gauss points, linear law) of a 32x8x8 beam"
    value = statistics.median(rates)
    nelem = tuple(int(x) for x in a.nelem.split(","))
    out = {
        "impl": "reference", "metric": "assembled elements/s (tangent+residual)", "value": value,
        "unit": "elements/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * np.prod(nelem) / value,
        "ms_per_step_note": "extrapolated: the whole beam's elements over the measured element rate of the "
                            "sample (the per-element cost does not depend on the mesh size)",
        "sample_seconds_per_step": sample_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"quadratic beam {nelem[0]}x{nelem[1]}x{nelem[2]} residual+tangent assembly, CPU",
                   "law": "linear strain gradient lambda=mu=1 ell=0.1", "sample": sample},
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": cores, "kind": "port",
                         "per_core": value / cores,
                         "sample": sample},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


# ------------------------------------------------------------------ GPU
def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    def __init__(self, path=None):
        self.samples = []
        self.proc = None
        self.path = path

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except OSError:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, dev=0):
        rows = [s for s in self.samples if len(s) >= 9 and s[0] == str(dev)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def bench_batched(ig, torch, dev, n, steps, warmup, flush, peaks):
    """Batched uneven instances: n seeded linear-law beams (nx in 8..64,
    ny = nz in 2..16, lambda, mu in [0.5, 2], length scale in [0.02, 0.2]),
    split-precision tangent (one persistent launch) + double-FP32 residual
    (one launch over every element and a gather per DOF) per assembly; schedule from the autotuner; one Newton step (assembly and
    GMRES cycles) replayed from CUDA graphs."""
    t0 = time.perf_counter()
    insts = ig.batch_instances(n, seed=SEED)
    B = ig.BatchAssembly(insts, law=ig.LAW_LINGRAD)
    t_init = time.perf_counter() - t0
    B.set_precision(ig.PREC_SPLIT)
    stream = torch.cuda.Stream(device=dev)
    B.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(SEED + 7)
    U = torch.tensor(rng.uniform(-1e-2, 1e-2, B.ndof), device=dev)
    RR = torch.zeros(B.ndof, dtype=torch.float64, device=dev)
    B.set_history(0, U)
    t0 = time.perf_counter()
    sched, t64, ttc = B.autotune(reps=2, frac=0.1)
    t_tune = time.perf_counter() - t0
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            B.assemble(U, RR, None)
    torch.cuda.synchronize()
    l0 = ig.launch_count()
    B.profile(True)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.fill_(float(k))
            evs[k][0].record(stream)
            B.assemble(U, RR, None)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    launches = ig.launch_count() - l0
    kinds = {kd: B.profile_read(kd) for kd in (0, 1)}
    B.profile(False)
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    ms_step = sum(ms) / steps
    tc_ms, tc_l, tc_e = kinds[1]
    res_ms, res_l, res_e = kinds[0]
    tc_ach = TAN_FLOP_PER_ELEM * tc_e / (tc_ms * 1e-3) / 1e12 if tc_ms > 0 else None
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    # one Newton step of the block-diagonal system from zero: assembly, then a
    # a fixed number of GMRES(100) iterations (Jacobi), replayed from CUDA graphs
    B.set_stream(None)
    Z = torch.zeros(B.ndof, dtype=torch.float64, device=dev)
    kits = 200
    opts = dict(snes_abstol=1e-300, ksp_rtol=1e-14, ksp_restart=100, ksp_max_it=kits, snes_max_it=1,
                use_graphs=1, pc=1, linesearch=0)
    F0 = torch.zeros_like(Z)
    B.residual(Z, F0)
    n0 = B.norms(F0)
    B.solve(Z.clone(), **opts)  # first call captures the graphs
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = B.solve(Z, **opts)
    B.synchronize()
    t_newton = time.perf_counter() - t0
    B.residual(Z, F0)
    n1 = B.norms(F0)
    red = n1 / np.maximum(n0, 1e-300)
    out = {"workload": f"{n} seeded uneven quadratic beams (nx 8..64, ny=nz 2..16), linear law with "
                       "per-instance lambda, mu in [0.5,2], ell in [0.02,0.2]; clamped x=0, traction 1e-3",
           "instances": n, "elements": B.nelem_total, "dof": B.ndof, "nnz": B.nnz,
           "precision": "split tangent (tcgen05 TF32x3, f32 accumulate) + " +
                        ("f64 residual" if os.environ.get("IGAPGPU_RES_DF", "1")[:1] == "0"
                         else "double-FP32 residual"),
           "value": B.nelem_total / (ms_step * 1e-3), "unit": "elements/s", "ms_per_step": ms_step,
           "step_ms": ms, "steps": steps, "gpu_launches_per_step": launches / steps,
           "tc_kernel_ms_per_step": tc_ms / steps, "residual_kernel_ms_per_step": res_ms / steps,
           "schedule": sched, "autotune_s": t_tune, "autotune_prefix_ms": {"fp64": t64, "tc": ttc},
           "init_s": t_init,
           "roofline": {"bound": "tensor", "kernel": "tc_tangent_kernel<batch>", "achieved": tc_ach,
                        "peak": bf16_peak, "unit": "TFLOP/s",
                        "frac": tc_ach / bf16_peak if tc_ach else None},
           "newton_step": {"seconds": t_newton, "newton_its": st["newton_its"], "ksp_its": st["ksp_its_total"],
                           "ms_per_ksp_it": None if not st["ksp_its_total"] else
                           1e3 * t_newton / st["ksp_its_total"],
                           "instance_residual_reduction": {"median": float(np.median(red)),
                                                           "max": float(np.max(red))},
                           "options": f"one Newton step from U=0: assembly then {kits} GMRES(100) MGS "
                                      "iterations with Jacobi, replayed from CUDA graphs"}}
    B.close()
    return out


PREDICTOR_FILE = os.path.join(ROOT, "igap4_gb300", "data", "predictor_gradelasttime.npz")


def bench_gradelast(ig, torch, nelem, steps, warmup, flush, cpu_seconds, cores):
    """The reference's own static law (gradelast, default material) assembled
    at `nelem`: residual + tangent per step in FP64 and in split precision,
    the split tangent's error against FP64, and the oracle port's rate for
    the same element kind on the host cores (a bounded sample, spawned
    processes started before this block's first GPU call)."""
    # the CPU sample first (spawned workers)
    n1, t1 = _cpu_worker_law((2, SEED))
    nel_cpu = max(2, min(int(cpu_seconds / (t1 / n1)), 16 * 4 * 4))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker_law, [(nel_cpu, SEED + i) for i in range(cores)])
    slowest = max(r[1] for r in res)
    cpu = {"value": sum(r[0] for r in res) / slowest, "unit": "elements/s", "cores": cores, "kind": "port",
           "per_core": nel_cpu / statistics.median([r[1] for r in res]),
           "sample": f"{cores} processes x {nel_cpu} elements (p=2, 64 points, gradelast) of a 16x4x4 beam; "
                     f"{slowest:.1f} s"}
    dev = torch.device("cuda")
    knots, w, X = ig.beam_mesh(nelem, LBEAM)
    bct, neu = ig.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_GRADELAST, bc_type=bct, neumann=neu)
    stream = torch.cuda.Stream(device=dev)
    A.set_stream(stream.cuda_stream)
    U = torch.tensor(np.random.default_rng(SEED).uniform(-1e-2, 1e-2, A.ndof), device=dev)
    RR = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    out = {"workload": f"quadratic beam {nelem[0]}x{nelem[1]}x{nelem[2]} ({A.nelem_total} elements), the "
                       "reference's static strain-gradient law (gradelast, default material), seeded uniform "
                       "state in [-1e-2, 1e-2]; one step = residual + tangent",
           "cpu_port": cpu}
    K64 = R64 = None
    for name, prec in (("fp64", ig.PREC_FP64), ("split", ig.PREC_SPLIT)):
        A.set_precision(prec)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                A.assemble(U, RR, None)
        torch.cuda.synchronize()
        ms = []
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.fill_(float(k))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                A.assemble(U, RR, None)
                e1.record(stream)
                ms.append((e0, e1))
        torch.cuda.synchronize()
        step_ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in ms)
        blk = {"ms_per_step": step_ms, "value": A.nelem_total / (step_ms * 1e-3), "unit": "elements/s",
               "vs_cpu_port": A.nelem_total / (step_ms * 1e-3) / cpu["value"]}
        K = torch.zeros(A.nnz, dtype=torch.float64, device=dev)
        R = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        A.tangent(U, K)  # on the context's stream: wait for it before torch reads K
        A.residual(U, R)
        A.synchronize()
        if K64 is None:
            K64, R64 = K, R
        else:
            blk["tangent_rel_err_vs_fp64"] = (torch.linalg.norm(K - K64) / torch.linalg.norm(K64)).item()
            blk["residual_rel_err_vs_fp64"] = (torch.linalg.norm(R - R64) / torch.linalg.norm(R64)).item()
            blk["precision"] = ("split tangent (law in FP32, TF32x3 contraction) + residual with the FP64 law "
                                "between double-FP32 interpolation and projection")
        out[name] = blk
    A.close()
    return out


def bench_transient(ig, torch, nelem, steps, start_steps=200, seed=9001, dt=5e-4):
    """Time to |F| <= 1e-8 per transient step, plain Newton from u_n against
    the learned predictor's guess (kept only when it lowers |F|): the
    reference's three-level law (gradelasttime, its default material, density
    1, its default time step 5e-4) on a quadratic beam clamped at x = 0 under a
    seeded tip-load history (sum of 4 sinusoids, amplitudes in [0, 1e-3],
    frequencies in [0.5, 5]) that the predictor never saw.  The first
    start_steps steps (plain Newton, not timed) carry the beam from rest into
    the regime where the default material transforms (the residual at u_n
    grows from 1e-6 to order 1); both arms then run the same `steps` steps
    from that state.  Newton: the FP64 law's residual (its inputs and
    projection in double-FP32 arithmetic), tangent on the tensor cores,
    GMRES(100) with cell-block Jacobi and two-pass classical Gram-Schmidt,
    replayed from CUDA graphs.  The step time is the wall time of the whole step
    (predictor, acceptance test, Newton)."""
    from igap4_gb300.train_predictor import load_network, transient_problem
    from igap4_gb300.transient import TipLoad, run_transient
    from igap4_gb300.predictor import LearnedPredictor

    A, _ = transient_problem(nelem, dt, prec="split")
    # cell-block Jacobi (2x2x2 control-point cells): on this law 72 against 166
    # GMRES iterations per step of scalar Jacobi, at a set-up of one 24x24
    # inversion per cell and Newton step
    opts = dict(snes_abstol=1e-8, ksp_rtol=1e-5, ksp_restart=100, ksp_max_it=5000, snes_max_it=30,
                use_graphs=1, pc=3, orth=1)
    load = TipLoad(seed=seed)
    t0 = time.perf_counter()
    _, warm = run_transient(A, load, start_steps, dt, opts=opts, record_states=False)
    start = run_transient.last
    t_warm = time.perf_counter() - t0

    def summary(recs):
        ms = np.array([1e3 * r.seconds for r in recs])
        return {"ms_per_step": float(ms.mean()), "ms_median": float(np.median(ms)),
                "newton_its_per_step": float(np.mean([r.newton_its for r in recs])),
                "gmres_its_per_step": float(np.mean([r.ksp_its for r in recs])),
                "fnorm_at_start_median": float(np.median([r.fnorm0 for r in recs])),
                "converged_all": bool(all(r.converged for r in recs)),
                "max_final_fnorm": float(max(r.fnorm for r in recs)),
                "prediction_used_fraction": float(np.mean([r.used_prediction for r in recs]))}

    _, plain = run_transient(A, load, steps, dt, opts=opts, record_states=False, start=start)
    out = {"workload": f"transient gradelasttime beam {nelem[0]}x{nelem[1]}x{nelem[2]} ({A.ndof} DOF), dt={dt}, "
                       f"steps {start_steps}..{start_steps + steps} of an unseen seeded tip-load history "
                       f"(seed {seed})",
           "tolerance": "Newton |F| <= 1e-8 (residual within 1e-12 of FP64)",
           "solver": "Newton, GMRES(100) rtol 1e-5 with two-pass classical Gram-Schmidt and cell-block "
                     "Jacobi (pc 3), cycles replayed from CUDA graphs",
           "plain": summary(plain),
           "warm_steps": {"steps": start_steps, "seconds": t_warm,
                          "all_converged": bool(all(r.converged for r in warm))}}
    if os.path.exists(PREDICTOR_FILE):
        net, sc = load_network(PREDICTOR_FILE, tuple(n + 2 for n in nelem))
        pred = LearnedPredictor(net, sc, A=A)
        pred(start[0], start[1], 0.0)  # first call: the network kernels' one-time set-up, not timed
        torch.cuda.synchronize()
        _, learned = run_transient(A, load, steps, dt, predictor=pred, opts=opts, record_states=False, start=start)
        out["learned"] = summary(learned)
        out["time_ratio_learned_vs_plain"] = out["learned"]["ms_per_step"] / out["plain"]["ms_per_step"]
        out["its_ratio_learned_vs_plain"] = (out["learned"]["newton_its_per_step"] /
                                             out["plain"]["newton_its_per_step"])
        z = np.load(PREDICTOR_FILE)
        out["predictor"] = {"file": os.path.relpath(PREDICTOR_FILE, ROOT), "training": json.loads(str(z["meta"])),
                            "inputs": str(z["mode"])}
        net.close()
    else:
        out["learned"] = None
        out["note"] = "no trained predictor file"
    A.close()
    return out


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    nelem = tuple(int(x) for x in a.nelem.split(","))

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        # spawn-based pool before any CUDA call
        cores = os.cpu_count() or 1
        r, nel, slowest, wall = cpu_rate(a.cpu_seconds, cores)
        cpu = {"value": r, "unit": "elements/s", "cores": cores, "kind": "port", "per_core": r / cores,
               "sample": f"{cores} concurrent single-threaded processes x {nel} elements each "
                         f"(residual+tangent, p=2, 64 points, linear law; oracle port of the "
                         f"reference loop) on a 32x8x8 beam; {slowest:.1f} s"}

    import torch
    import igap4_gb300 as ig
    from igap4_gb300.replicas import job_rate, max_over_ranks

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    bct, neu = ig.clamp_bc((0,), 1, (0.0, 0.0, -1e-3))
    knots, w, X = ig.beam_mesh(nelem, LBEAM)
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_LINGRAD, par=LAW_PAR, bc_type=bct, neumann=neu)
    stream = torch.cuda.Stream(device=dev)
    A.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(SEED + rank)
    U = torch.tensor(rng.uniform(-1e-2, 1e-2, A.ndof), device=dev)
    RR = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device=dev)

    def step():
        A.assemble(U, RR, None)  # residual + tangent into the context matrix

    def measure(prec, steps, warmup):
        A.set_precision(prec)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                step()
        torch.cuda.synchronize()
        launches0 = ig.launch_count()
        A.profile(True)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.fill_(float(k))  # L2 flush, outside the events
                evs[k][0].record(stream)
                step()
                evs[k][1].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        launches = ig.launch_count() - launches0
        kinds = {kd: A.profile_read(kd) for kd in (0, 1)}
        A.profile(False)
        step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
        dev_ms = max_over_ranks(sum(step_ms), dev)
        return dev_ms / steps, step_ms, kinds, launches

    sampler = ClockSampler()
    sampler.start()
    t_wall0 = time.perf_counter()
    precs = {"fp64q": ig.PREC_OZAKI, "fp64": ig.PREC_FP64, "split": ig.PREC_SPLIT}
    head = "fp64q" if a.prec == "all" else a.prec
    prep_launches = {}

    def prepare(name):
        # a mode's one-time set-up (BF16 slices, cached Gram operands), outside the timing
        n0 = ig.launch_count()
        A.set_precision(precs[name])
        prep_launches[name] = ig.launch_count() - n0

    prepare(head)
    runs = {head: measure(precs[head], a.steps, a.warmup)}
    t_wall = time.perf_counter() - t_wall0
    ms_per_step, step_ms, kinds, launches = runs[head]
    value = job_rate(A.nelem_total, ms_per_step, world)
    dev_ms = ms_per_step * a.steps
    others = [m for m in ("fp64q", "fp64", "split") if m != head] if a.prec == "all" else []
    for name in others:
        prepare(name)
        runs[name] = measure(precs[name], a.steps, max(1, a.warmup - 1))
    # tangent and residual error of each mode against the FP64 kernels, at full size
    A.set_precision(ig.PREC_FP64)
    K64 = torch.zeros(A.nnz, dtype=torch.float64, device=dev)
    R64 = torch.zeros(A.ndof, dtype=torch.float64, device=dev)
    Kx, Rx = torch.zeros_like(K64), torch.zeros_like(R64)
    torch.cuda.synchronize()  # the library writes them on the context's stream
    A.tangent(U, K64)
    A.residual(U, R64)
    errs, rerrs = {"fp64": 0.0}, {"fp64": 0.0}
    for name in runs:
        if name == "fp64":
            continue
        A.set_precision(precs[name])
        A.tangent(U, Kx)
        A.residual(U, Rx)
        A.synchronize()
        errs[name] = (torch.linalg.norm(Kx - K64) / torch.linalg.norm(K64)).item()
        rerrs[name] = (torch.linalg.norm(Rx - R64) / torch.linalg.norm(R64)).item()
    del K64, Kx, R64, Rx
    A.set_precision(precs[head])

    # e2e through the C ABI with pinned host buffers
    Uh = torch.empty(A.ndof, dtype=torch.float64, pin_memory=True)
    Uh.copy_(U.cpu())
    RRh = torch.empty(A.ndof, dtype=torch.float64, pin_memory=True)
    e2e_ms = []
    for k in range(max(2, min(a.steps, 5))):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        A.assemble(Uh.numpy(), RRh.numpy(), None)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = world * A.nelem_total / (statistics.median(e2e_ms) * 1e-3)

    # SpMV of the assembled matrix (the MATSHELL multiply), FP64
    x = torch.tensor(rng.standard_normal(A.ndof), device=dev)
    y = torch.zeros_like(x)
    with torch.cuda.stream(stream):
        for _ in range(5):
            A.matmult(x, y)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.spmv):
            A.matmult(x, y)
        e1.record(stream)
    torch.cuda.synchronize()
    spmv_ms = e0.elapsed_time(e1) / max(a.spmv, 1)
    # the structured multiply streams the values (8 B per nonzero; the column
    # of each entry is computed from the stencil), the row offsets, x and y
    spmv_bytes = A.nnz * 8 + (A.ndof + 1) * 8 + 2 * A.ndof * 8
    sampler.stop()

    peaks = _peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    fp64_peak = ig.measure_fp64_peak()
    fp32_peak = ig.measure_fp32_peak()
    nelem_total, ndof_total, nnz_total = A.nelem_total, A.ndof, A.nnz
    A.close()  # frees the beam's matrix and geometry cache before the batched workload
    del x, y
    batched = None
    if a.batch > 0:
        sampler.start()
        batched = bench_batched(ig, torch, dev, a.batch, a.batch_steps, max(3, a.warmup), flush, peaks)
        sampler.stop()
    gradelast = None
    if a.gradelast_nelem != "0" and world == 1:
        sampler.start()
        gradelast = bench_gradelast(ig, torch, tuple(int(v) for v in a.gradelast_nelem.split(",")), a.steps,
                                    max(3, a.warmup), flush, 2.0, os.cpu_count() or 1)
        sampler.stop()
    transient = None
    if a.transient_steps > 0 and world == 1:
        transient = bench_transient(ig, torch, tuple(int(v) for v in a.transient_nelem.split(",")),
                                    a.transient_steps)

    def fp64_roofline(name, kms, kl, kc, step_total_ms):
        """The FP64 element kernel of a mode (fused residual + tangent in the
        FP64 mode, residual only in the tensor-core modes)."""
        fused = name == "fp64"
        per_launch_ms = kms / max(kl, 1)
        alg = (TAN_FLOP_PER_ELEM + RES_FLOP_PER_ELEM) if fused else RES_FLOP_PER_ELEM
        exe = EXEC_FLOP_FP64_ELEM if fused else EXEC_FLOP_RES_ELEM
        ach = alg * kc / max(kl, 1) / (per_launch_ms * 1e-3) / 1e12
        ex_ach = exe * kc / max(kl, 1) / (per_launch_ms * 1e-3) / 1e12
        out = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
               "executed_flop_per_element": exe, "executed_achieved": ex_ach, "executed_frac": ex_ach / fp64_peak,
               "kernel": "element_kernel (fused residual+tangent, FP64)" if fused else
                         "element_kernel (residual, FP64)",
               "peak_source": "measured in-run FP64 FMA throughput (MEASURED_PEAKS.json has no FP64 figure)",
               "algorithmic_flop_per_element": alg, "elements_per_launch": kc / max(kl, 1),
               "avg_launch_ms": per_launch_ms,
               "kernel_share_of_step": kms / step_total_ms if step_total_ms > 0 else None,
               "traffic": (TRAFFIC_FP64_ELEM * kc / max(kl, 1)) if fused else None}
        if fused:
            out["frac_note"] = ("achieved counts the dense R^T D R FLOPs per element; the kernel evaluates the "
                                "same sum through Gram sums with 5.3x fewer FLOPs, so frac exceeds 1; "
                                "executed_frac is the FP64 pipe fraction")
        return out

    def res_df_roofline(kms, kl, kc, step_total_ms):
        """The double-FP32 residual kernel of the tensor-core modes: bound by the
        FP32 pipe (lane instructions against the measured FMA issue rate)."""
        per_launch_ms = kms / max(kl, 1)
        per_launch_el = kc / max(kl, 1)
        sec = per_launch_ms * 1e-3
        ach = EXEC_F32_RES_DF_ELEM * per_launch_el / sec / 1e12
        peak = fp32_peak / 2  # FMA issue rate: one lane instruction per FMA (2 FLOP)
        gbs = ALG_BYTES_RES_DF_ELEM * per_launch_el / sec / 1e9
        return {"bound": "fp32", "kernel": "res_df_kernel (linear-law residual in double-FP32 arithmetic: "
                                          "pair cache, compensated dot products, a thread per Gauss point)",
                "achieved": ach, "peak": peak, "unit": "T FP32-pipe lane instructions/s", "frac": ach / peak,
                "executed_fp32_instructions_per_element": EXEC_F32_RES_DF_ELEM,
                "peak_source": "measured in-run FP32 FMA throughput / 2 (MEASURED_PEAKS.json has no FP32 figure)",
                "fp32_fma_tflops_measured": fp32_peak,
                "fp64_equivalent_tflops": RES_FLOP_PER_ELEM * per_launch_el / sec / 1e12,
                "fp64_equivalent_note": "the residual's FP64 FLOPs per element / kernel time: "
                                        "against the FP64 pipe's measured peak",
                "fp64_peak": fp64_peak,
                "hbm_algorithmic_bytes_per_element": ALG_BYTES_RES_DF_ELEM, "hbm_achieved_gbs": gbs,
                "hbm_frac": gbs / hbm_peak, "traffic": TRAFFIC_RES_DF_ELEM * per_launch_el,
                "avg_launch_ms": per_launch_ms, "elements_per_launch": per_launch_el,
                "kernel_share_of_step": kms / step_total_ms if step_total_ms > 0 else None}

    def tc_roofline(name, kms, kl, kc):
        per_launch_ms = kms / max(kl, 1)
        per_launch_el = kc / max(kl, 1)
        if name == "split":
            exe, kern = EXEC_FLOP_TC_ELEM, ("tcw_kernel (cached sqrt(w)-weighted Gram operands, warp-specialised "
                                           "copy/split/MMA/scatter; tcgen05.mma kind::tf32, TF32x3)")
            bytes_el, traffic = ALG_BYTES_TCS_ELEM, TRAFFIC_TCS_ELEM * per_launch_el
        else:
            exe, kern = EXEC_FLOP_OZ_ELEM, ("tco_kernel (error-free BF16 slices of the Gram operands, one bulk "
                                           "copy per chunk, 24 tcgen05.mma kind::f16 per chunk into 4 TMEM "
                                           "accumulators; a thread per basis pair recombines its 3x3 block of "
                                           "G with FP32 error-free sums and adds K at (b,c) and (c,b))")
            bytes_el, traffic = ALG_BYTES_OZ_ELEM, TRAFFIC_OZ_ELEM * per_launch_el
        gbs = bytes_el * per_launch_el / (per_launch_ms * 1e-3) / 1e9
        ex_ach = exe * per_launch_el / (per_launch_ms * 1e-3) / 1e12
        return {"bound": "hbm", "kernel": kern, "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": gbs / hbm_peak, "hbm_algorithmic_bytes_per_element": bytes_el,
                "traffic": traffic, "executed_tensor_flop_per_element": exe,
                "executed_tensor_tflops": ex_ach, "executed_tensor_frac_of_bf16": ex_ach / bf16_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy) and bf16_tflops",
                "avg_launch_ms": per_launch_ms, "elements_per_launch": per_launch_el}

    mode_desc = {"fp64q": "double-FP32 residual (FP32 pipe); tangent on the tensor cores from error-free BF16 "
                          "slices (FP64 quality)",
                 "fp64": "FP64 residual and tangent (FP64 pipe)",
                 "split": "double-FP32 residual (FP32 pipe); TF32x3 tensor-core tangent"}
    blocks = {}
    for name, (mms, mstep, mkinds, mlaunch) in runs.items():
        res_ms, res_l, res_c = mkinds[0]
        tc_ms, tc_l, tc_c = mkinds[1]
        tot = mms * a.steps
        b = {"value": world * nelem_total / (mms * 1e-3), "unit": "elements/s", "ms_per_step": mms,
             "step_ms": mstep, "gpu_launches": mlaunch, "precision": mode_desc[name],
             "tangent_rel_err_vs_fp64": errs.get(name), "residual_rel_err_vs_fp64": rerrs.get(name),
             "setup_launches": prep_launches.get(name)}
        if name == "fp64":
            b["fp64_kernel_ms_per_step"] = res_ms / a.steps
            b["fp64_kernel_roofline"] = fp64_roofline(name, res_ms, res_l, res_c, tot)
        else:
            b["res_kernel_ms_per_step"] = res_ms / a.steps
            b["res_kernel_roofline"] = res_df_roofline(res_ms, res_l, res_c, tot)
            b["tc_kernel_ms_per_step"] = tc_ms / a.steps
            if tc_l > 0:
                b["tc_kernel_roofline"] = tc_roofline(name, tc_ms, tc_l, tc_c)
        blocks[name] = b
    hb = blocks[head]
    # the headline's roofline: its dominant kernel
    if head == "fp64":
        roofline = hb["fp64_kernel_roofline"]
    elif "tc_kernel_roofline" in hb and hb["tc_kernel_ms_per_step"] > hb["res_kernel_ms_per_step"]:
        roofline = hb["tc_kernel_roofline"]
    else:
        roofline = hb["res_kernel_roofline"]
    if rank == 0:
        out = {
            "metric": "assembled elements/s (tangent+residual)", "value": value, "unit": "elements/s",
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64q": "f64-quality (residual: f32 pairs; tangent: bf16 slices, exact f32 accumulation, "
                               "f32-pair recombination; f64 global accumulation)",
                      "fp64": "f64", "split": "tf32x3/f32-acc tangent, f32-pair residual"}[head],
            "data": "synthetic",
            "config": {"workload": f"quadratic beam {nelem[0]}x{nelem[1]}x{nelem[2]} "
                                   f"({nelem_total} elements, {ndof_total} DOF, nnz {nnz_total}) "
                                   "residual Vec + CSR tangent assembly",
                       "law": "linear isotropic strain gradient lambda=1 mu=1 ell=0.1",
                       "quadrature": "4x4x4 Gauss", "bc": "clamped x=0, traction 1e-3 in -z at x=4",
                       "state": "seeded uniform [-1e-2,1e-2] per DOF",
                       "precision": mode_desc[head],
                       "tangent_rel_err_vs_fp64": errs.get(head),
                       "residual_rel_err_vs_fp64": rerrs.get(head),
                       "l2": "flushed (256 MiB write) before every timed step; the 1.25 GB CSR output also exceeds L2",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "elements/s", "h2d_bytes_per_step": ndof_total * 8,
                    "d2h_bytes_per_step": ndof_total * 8,
                    "note": "state H2D from pinned host memory, residual D2H; tangent kept in the device matrix"},
            "gpu_launches": launches,
            "roofline": roofline,
            "spmv": {"ms": spmv_ms, "GB_per_s": spmv_bytes / (spmv_ms * 1e-3) / 1e9,
                     "frac_of_hbm": spmv_bytes / (spmv_ms * 1e-3) / 1e9 / hbm_peak, "bytes": spmv_bytes,
                     "repetitions": a.spmv,
                     # one FP64 FMA per nonzero: on this GPU the FP64 pipe, not HBM, bounds the multiply
                     "fp64_tflops": 2 * nnz_total / (spmv_ms * 1e-3) / 1e12,
                     "frac_of_fp64": 2 * nnz_total / (spmv_ms * 1e-3) / 1e12 / fp64_peak,
                     "bound": "fp64"},
            "cpu_baseline": cpu,
            "modes": blocks,
            "batched": batched,
            "gradelast": gradelast,
            "transient": transient,
            "clocks": sampler.summary(local),
            "step_ms": step_ms,
            "wall_s": t_wall,
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

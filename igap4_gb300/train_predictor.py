"""Train the learned Newton predictor on trajectories of the plain method and
measure what it gains (the transient beam of the learned-predictor workload,
scaled to the sizes given on the command line).

    python -m igap4_gb300.train_predictor --nelem 16,4,4 --train 6 --steps 60 --test 2

1. Plain-method trajectories (transient law, seeded tip loads) on the device.
2. Samples (u_n, u_{n-1}, load increment) -> correction to linear extrapolation.
3. Adam training with the library's own BF16 network kernels.
4. Unseen load histories: Newton iterations and wall time per step, plain
   Newton (guess u_n) vs the predictor (kept only when it lowers |F|).
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np


def transient_problem(nelem, dt=1e-2, rho=1.0, prec="fp64"):
    """The transient beam of the learned-predictor workload: the reference's
    three-level law (gradelasttime, default material, density rho, time step
    dt), clamped at x = 0; prec "split" puts the Newton tangent on the tensor
    cores (the residual keeps the FP64 law, its interpolation and projection
    in double-FP32 arithmetic within 1e-12 of FP64, so the converged states
    agree with an FP64 Newton to its tolerance)."""
    import igap4_gb300 as ig

    par = np.array(ig.LAW_DEFAULT_PAR[ig.LAW_GRADELASTTIME], dtype=float)
    par[5], par[7] = rho, dt
    bct, _ = ig.clamp_bc((0,))
    knots, w, X = ig.beam_mesh(nelem, (4.0, 1.0, 1.0))
    A = ig.Assembly(nelem, knots, w, X, law=ig.LAW_GRADELASTTIME, par=par, bc_type=bct)
    A.set_precision(ig.PREC_SPLIT if prec == "split" else ig.PREC_FP64)
    return A, par


def generate(A, seeds, nsteps, dt, amax, opts=None):
    from .transient import TipLoad, run_transient

    trajs = []
    for s in seeds:
        load = TipLoad(seed=int(s), amax=amax)
        states, recs = run_transient(A, load, nsteps, dt, opts=opts)
        loads = np.array([0.0] + [load.value((n + 1) * dt) for n in range(nsteps)])
        trajs.append((states, loads, recs, load))
        print(f"trajectory {s}: {nsteps} steps, {np.mean([r.newton_its for r in recs]):.2f} Newton its/step, "
              f"all converged {all(r.converged for r in recs)}", file=sys.stderr, flush=True)
    return trajs


def build_dataset(trajs):
    from .predictor import make_samples

    X, Y = [], []
    for states, loads, _, _ in trajs:
        x, y = make_samples(states, loads, None)
        X += x
        Y += y
    return X, Y


def residual_inputs(A, trajs, dt):
    """For every sample of build_dataset (same order): the residual of the
    step's equations at the extrapolation 2 u_n - u_{n-1}, with the history
    levels and the load of that step (what the transient driver sees when it
    asks the predictor)."""
    R = []
    for states, _, _, load in trajs:
        for n in range(1, len(states) - 1):
            A.set_history(1, np.ascontiguousarray(states[n]))
            A.set_history(2, np.ascontiguousarray(states[n - 1]))
            A.set_neumann(load.table((n + 1) * dt))
            R.append(A.residual(np.ascontiguousarray(2.0 * states[n] - states[n - 1])).copy())
    return R


def train(A, X, Y, epochs=40, batch=8, lr=2e-3, seed=0, storage="bf16", log=None, R=None, relative=False):
    """Adam on the samples; R (residual inputs, residual_inputs()) selects
    the residual-input network, relative=True the step-relative one, else the
    load-increment input."""
    import torch

    from .predictor import ConvNet, Scales, features

    lattice = tuple(n + 2 for n in A.nelem)
    su = max(1e-30, max(np.abs(x[0]).max() for x in X))
    if relative:  # targets in units of each sample's largest increment component
        sd = [max(1e-300, np.abs(x[0] - x[1]).max()) for x in X]
        Y = [y / s for y, s in zip(Y, sd)]
    so = max(1e-30, max(np.abs(y).max() for y in Y))
    if relative:
        scales = Scales(u=su, load=max(1e-30, max(np.abs(x[2]).max() for x in X)), out=so, mode="relative")
        thirds = [x[2] for x in X]
    elif R is not None:
        scales = Scales(u=su, load=max(1e-30, max(np.abs(r).max() for r in R)), out=so, mode="residual")
        thirds = R
    else:
        scales = Scales(u=su, load=max(1e-30, max(np.abs(x[2]).max() for x in X)), out=so)
        thirds = [x[2] for x in X]
    P = int(np.prod(lattice))
    dev = torch.device("cuda")
    feats = torch.stack([features(torch.tensor(x[0], device=dev), torch.tensor(x[1], device=dev),
                                  torch.tensor(t, device=dev) if R is not None else t, scales)
                         for x, t in zip(X, thirds)])
    targ = torch.stack([torch.tensor(y / so, dtype=torch.float32, device=dev).view(P, 3) for y in Y])
    net = ConvNet(lattice, batch_max=batch, storage=storage, seed=seed)
    rng = np.random.default_rng(seed)
    n = len(X)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for i in range(0, n - batch + 1, batch):
            idx = torch.tensor(order[i:i + batch], device=dev)
            tot += net.train_step(feats[idx].contiguous(), targ[idx].contiguous(), lr) * batch
        hist.append(tot / max(1, (n // batch) * batch))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return net, scales, hist


def eval_starts(A, seeds, n0, dt, amax, opts=None):
    """Per seed, the state after n0 plain steps from rest: (u_n, u_{n-1}, n0),
    so that the arms of an evaluation are timed on the same later window."""
    from .transient import TipLoad, run_transient

    out = {}
    for s in seeds:
        if n0 <= 0:
            out[int(s)] = None
            continue
        run_transient(A, TipLoad(seed=int(s), amax=amax), n0, dt, opts=opts, record_states=False)
        out[int(s)] = run_transient.last
    return out


def evaluate(A, seeds, nsteps, dt, amax, predictor=None, opts=None, starts=None):
    from .transient import TipLoad, run_transient

    its, times, used = [], [], []
    for s in seeds:
        load = TipLoad(seed=int(s), amax=amax)
        _, recs = run_transient(A, load, nsteps, dt, predictor=predictor, opts=opts, record_states=False,
                                start=(starts or {}).get(int(s)))
        its += [r.newton_its for r in recs]
        times += [r.seconds for r in recs]
        used += [r.used_prediction for r in recs]
    return {"newton_its_per_step": float(np.mean(its)), "seconds_per_step": float(np.mean(times)),
            "prediction_used_fraction": float(np.mean(used)) if predictor else 0.0}


def save_network(path, net, scales, meta=None):
    """Trained parameters (FP32 master copy) and input/output scales."""
    np.savez(path, params=net.get_params(), scale_u=scales.u, scale_load=scales.load, scale_out=scales.out,
             mode=scales.mode, meta=json.dumps(meta or {}))


def load_network(path, lattice, batch_max=1, storage="bf16"):
    """(ConvNet on `lattice`, Scales) from a file written by save_network;
    the network is convolutional, so any lattice size takes the weights."""
    from .predictor import ConvNet, Scales

    z = np.load(path, allow_pickle=False)
    sc = Scales(u=float(z["scale_u"]), load=float(z["scale_load"]), out=float(z["scale_out"]), mode=str(z["mode"]))
    return ConvNet(lattice, batch_max=batch_max, storage=storage, params=z["params"]), sc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nelem", default="16,4,4")
    ap.add_argument("--train", type=int, default=6, help="training trajectories")
    ap.add_argument("--test", type=int, default=2, help="unseen evaluation trajectories")
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--dt", type=float, default=1e-2)
    ap.add_argument("--amax", type=float, default=1e-3)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--eval-nelem", default=None, help="evaluate on another mesh (default: same)")
    ap.add_argument("--features", default="load", choices=["load", "residual", "both", "relative"],
                    help="network inputs: load increment, residual at the extrapolation, or the step-relative "
                         "form (last increment and correction in units of the sample's largest increment)")
    ap.add_argument("--compare-shortened", action="store_true",
                    help="also evaluate the best of the guess and two shortened steps along its correction")
    ap.add_argument("--prec", default="fp64", choices=["fp64", "split"], help="Newton tangent precision")
    ap.add_argument("--save", default=None, help="write the trained network (params, scales) to this .npz")
    ap.add_argument("--eval-start", type=int, default=0,
                    help="plain steps from rest before the evaluated window (not timed)")
    ap.add_argument("--eval-steps", type=int, default=None, help="evaluated steps (default --steps)")
    a = ap.parse_args()
    import torch  # noqa: F401

    from .predictor import LearnedPredictor

    nelem = tuple(int(v) for v in a.nelem.split(","))
    opts = dict(snes_abstol=1e-8, ksp_rtol=1e-5, ksp_restart=100, ksp_max_it=5000, snes_max_it=30, use_graphs=1,
                orth=1)
    A, _ = transient_problem(nelem, a.dt, prec=a.prec)
    t0 = time.perf_counter()
    trajs = generate(A, range(1000, 1000 + a.train), a.steps, a.dt, a.amax, opts)
    t_gen = time.perf_counter() - t0
    X, Y = build_dataset(trajs)
    modes = ["load", "residual"] if a.features == "both" else [a.features]
    R = residual_inputs(A, trajs, a.dt) if "residual" in modes else None
    nets, t_train = {}, {}
    for mode in modes:
        t0 = time.perf_counter()
        nets[mode] = train(A, X, Y, epochs=a.epochs, R=R if mode == "residual" else None,
                           relative=mode == "relative", log=lambda msg: print(msg, file=sys.stderr, flush=True))
        t_train[mode] = time.perf_counter() - t0
    if a.eval_nelem:
        A.close()
        A, _ = transient_problem(tuple(int(v) for v in a.eval_nelem.split(",")), a.dt, prec=a.prec)
        from .predictor import ConvNet

        lattice = tuple(n + 2 for n in A.nelem)
        nets = {m: (ConvNet(lattice, batch_max=1, storage="bf16", params=net.get_params()), sc, h)
                for m, (net, sc, h) in nets.items()}
    if a.save:
        net, sc, hist = nets[modes[-1]]
        save_network(a.save, net, sc, meta={"train_mesh": list(nelem), "train_trajectories": a.train,
                                            "steps": a.steps, "epochs": a.epochs, "dt": a.dt, "amax": a.amax,
                                            "loss_first": hist[0], "loss_last": hist[-1]})
    seeds = range(5000, 5000 + a.test)
    ev_steps = a.eval_steps or a.steps
    starts = eval_starts(A, seeds, a.eval_start, a.dt, a.amax, opts)
    plain = evaluate(A, seeds, ev_steps, a.dt, a.amax, None, opts, starts)
    from .predictor import ConvNet, Scales, init_params

    extrap_net = ConvNet(tuple(n + 2 for n in A.nelem), batch_max=1, storage="bf16", params=init_params(0))
    extrap = evaluate(A, seeds, ev_steps, a.dt, a.amax, LearnedPredictor(extrap_net, Scales(), scaled=False), opts,
                      starts)
    out = {"train_mesh": list(nelem), "eval_mesh": list(A.nelem), "train_trajectories": a.train,
           "steps": a.steps, "dt": a.dt, "eval_window": [a.eval_start, a.eval_start + ev_steps],
           "samples": len(X), "generation_s": t_gen, "plain": plain, "extrapolation_only": extrap}
    for mode, (net, scales, hist) in nets.items():
        learned = evaluate(A, seeds, ev_steps, a.dt, a.amax, LearnedPredictor(net, scales, A=A), opts, starts)
        key = "learned" if mode == modes[-1] else f"learned_{mode}"
        out[key] = learned
        out[key + "_training"] = {"inputs": mode, "seconds": t_train[mode], "loss_first": hist[0],
                                  "loss_last": hist[-1]}
        if a.compare_shortened:
            out[key + "_best_of_shortened"] = evaluate(A, seeds, ev_steps, a.dt, a.amax,
                                                       LearnedPredictor(net, scales, scaled=True, A=A), opts, starts)
    out["time_ratio_learned_vs_plain"] = out["learned"]["seconds_per_step"] / plain["seconds_per_step"]
    out["its_ratio_learned_vs_plain"] = out["learned"]["newton_its_per_step"] / plain["newton_its_per_step"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""Learned Newton predictor for the transient runs (no counterpart in the
reference; an addition to its solver path).

A 3-D convolutional network on the control-point lattice predicts the next
displacement increment.  It is a correction to linear extrapolation
u_ext = u_n + (u_n - u_{n-1}),

    guess = u_ext + s_out * net([u_n / s_u, u_{n-1} / s_u, c / s_c]),

where the third input block c is either the load increment (the same vector
at every point) or the residual F(u_ext) of the step's equations at the
extrapolation (per point: what Newton's first correction would remove), and
the last layer starts at zero, so an untrained network reproduces the
extrapolation.  The network's forward, backward and Adam step are the
library's own kernels (igapgpu_net_*); torch is used here only to hold device
buffers and to pack the 9 input channels.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _check, _ptr, lib

CIN = (9, 32, 32, 32)
COUT = (32, 32, 32, 3)
NPARAM = sum(co * 27 * ci for ci, co in zip(CIN, COUT)) + sum(COUT)


def _bind():
    L = lib()
    if getattr(L, "_net_bound", False):
        return L
    vp = ctypes.c_void_p
    L.igapgpu_net_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int]
    L.igapgpu_net_destroy.argtypes = [vp]
    L.igapgpu_net_num_params.argtypes = [vp]
    L.igapgpu_net_num_params.restype = ctypes.c_int64
    L.igapgpu_net_set_stream.argtypes = [vp, vp]
    for f in ("igapgpu_net_set_params", "igapgpu_net_get_params", "igapgpu_net_get_grads"):
        getattr(L, f).argtypes = [vp, vp]
    L.igapgpu_net_forward.argtypes = [vp, vp, vp, ctypes.c_int]
    L.igapgpu_net_train_step.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_float,
                                         ctypes.POINTER(ctypes.c_float)]
    L._net_bound = True
    return L


def init_params(seed: int, zero_last: bool = True) -> np.ndarray:
    """He-normal weights for the ReLU layers; the output layer starts at zero."""
    rng = np.random.default_rng(seed)
    ws = []
    for l, (ci, co) in enumerate(zip(CIN, COUT)):
        std = np.sqrt(2.0 / (27 * ci))
        w = rng.standard_normal((co, 27, ci)) * std
        if l == 3 and zero_last:
            w[:] = 0.0
        ws.append(w.ravel())
    bs = [np.zeros(co) for co in COUT]
    return np.concatenate(ws + bs).astype(np.float32)


class ConvNet:
    """Device network over a lattice (nx, ny, nz); storage 'bf16' or 'f32'."""

    def __init__(self, lattice, batch_max=1, storage="bf16", params=None, seed=0):
        L = _bind()
        h = ctypes.c_void_p()
        _check(L.igapgpu_net_create(ctypes.byref(h), int(lattice[0]), int(lattice[1]), int(lattice[2]),
                                    int(batch_max), 1 if storage == "bf16" else 0))
        self.h = h
        self.lattice = tuple(int(v) for v in lattice)
        self.P = int(np.prod(self.lattice))
        self.batch_max = batch_max
        self.set_params(init_params(seed) if params is None else params)

    def close(self):
        if getattr(self, "h", None):
            lib().igapgpu_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == NPARAM
        _check(lib().igapgpu_net_set_params(self.h, _ptr(p)))

    def get_params(self):
        p = np.zeros(NPARAM, np.float32)
        _check(lib().igapgpu_net_get_params(self.h, _ptr(p)))
        return p

    def get_grads(self):
        g = np.zeros(NPARAM, np.float32)
        _check(lib().igapgpu_net_get_grads(self.h, _ptr(g)))
        return g

    def forward(self, x, out):
        """x: CUDA float32 [B, P, 9]; out: CUDA float32 [B, P, 3]."""
        _check(lib().igapgpu_net_forward(self.h, _ptr(x), _ptr(out), int(x.shape[0])))
        return out

    def train_step(self, x, target, lr):
        loss = ctypes.c_float()
        _check(lib().igapgpu_net_train_step(self.h, _ptr(x), _ptr(target), int(x.shape[0]), float(lr),
                                            ctypes.byref(loss)))
        return float(loss.value)


@dataclass
class Scales:
    u: float = 1.0
    load: float = 1.0   # scale of the third input block (load increment or residual)
    out: float = 1.0
    # "load": inputs u_n, u_{n-1}, load increment; "residual": u_n, u_{n-1},
    # F(u_ext); "relative": u_n, the last increment u_n - u_{n-1} and the load
    # increment, the increment and the output measured in units of the
    # sample's own largest increment component (the state of a transforming
    # material grows by orders of magnitude along a trajectory)
    mode: str = "load"


def features(u_n, u_nm1, third, scales: Scales):
    """[P, 9] float32 input channels from device DOF vectors (3 per point);
    third: the load increment (3 values) or a residual DOF vector."""
    import torch

    P = u_n.numel() // 3
    x = torch.empty((P, 9), dtype=torch.float32, device=u_n.device)
    x[:, 0:3] = (u_n.view(P, 3) / scales.u).float()
    if scales.mode == "relative":
        inc = u_n - u_nm1
        x[:, 3:6] = (inc / step_scale(inc)).view(P, 3).float()
    else:
        x[:, 3:6] = (u_nm1.view(P, 3) / scales.u).float()
    if scales.mode == "residual":
        x[:, 6:9] = (torch.as_tensor(third, device=u_n.device).view(P, 3) / scales.load).float()
    else:
        x[:, 6:9] = torch.as_tensor(np.asarray(third, np.float32) / scales.load, device=u_n.device)
    return x


def step_scale(inc):
    """The largest component of a state increment (a device scalar), 1e-300 at rest."""
    import torch

    return torch.clamp(inc.abs().max(), min=1e-300)


class LearnedPredictor:
    """Callable (u_n, u_{n-1}, dload) -> guess for u_{n+1} (device float64)."""

    def __init__(self, net: ConvNet, scales: Scales, dload_dir=(0.0, 0.0, 1.0), scaled: bool = False, A=None):
        import torch

        if scales.mode == "residual" and A is None:
            raise ValueError("a residual-input predictor needs the Assembly (A=...)")
        self.A = A
        self.scaled = scaled
        self.net = net
        self.scales = scales
        self.dir = np.asarray(dload_dir, np.float64)
        self.out = torch.empty((1, net.P, 3), dtype=torch.float32, device="cuda")
        self.F = None

    def correction(self, u_n, u_nm1, dload_scalar):
        if self.scales.mode == "residual":
            # residual of this step's equations (history levels and load set by
            # the transient driver) at the extrapolation
            if self.F is None or self.F.numel() != u_n.numel():
                import torch

                self.F = torch.zeros_like(u_n)
            self.A.residual((u_n + (u_n - u_nm1)).contiguous(), self.F)
            x = features(u_n, u_nm1, self.F, self.scales)[None]
        else:
            x = features(u_n, u_nm1, self.dir * dload_scalar, self.scales)[None]
        self.net.forward(x, self.out)
        corr = self.out.view(-1).double() * self.scales.out
        if self.scales.mode == "relative":
            corr = corr * step_scale(u_n - u_nm1)
        return corr

    def __call__(self, u_n, u_nm1, dload_scalar):
        return u_n + (u_n - u_nm1) + self.correction(u_n, u_nm1, dload_scalar)

    def candidates(self, u_n, u_nm1, dload_scalar):
        """The network's guess and, with scaled=True, two shortened steps
        along its correction (half of it, none: the linear extrapolation); the
        transient driver keeps the one with the smallest residual, or u_n.
        Measured on a 16x4x4 beam (16 training trajectories of 40 steps, 2
        unseen load histories): the shortened steps often have the smaller
        residual but need more Newton iterations (1.95 per step against 1.78
        for the network's guess alone), so they are off by default."""
        ext = u_n + (u_n - u_nm1)
        corr = self.correction(u_n, u_nm1, dload_scalar)
        return [ext + corr, ext + 0.5 * corr, ext] if self.scaled else [ext + corr]


def make_samples(states, loads, lattice_points):
    """Training pairs from one trajectory: inputs (u_n, u_{n-1}, dload) and
    targets = (u_{n+1} - u_n) - (u_n - u_{n-1}) for n = 1 .. N-1."""
    X, Y = [], []
    for n in range(1, len(states) - 1):
        un, unm1, unp1 = states[n], states[n - 1], states[n + 1]
        dl = np.array([0.0, 0.0, loads[n + 1] - loads[n]])
        X.append((un, unm1, dl))
        Y.append((unp1 - un) - (un - unm1))
    return X, Y


def time_convolutions(lattice=(66, 18, 18), batch=8, reps=10, seed=0):
    """Wall-clock ms of one forward pass and one training step (forward, MSE,
    backward, Adam) of a BF16 network, with the tensor-core convolutions
    (IGAPGPU_NET_TC=1) and with the scalar kernels (=0), on the same seeded
    network and inputs; 3 warm-up repetitions, synchronised."""
    import os
    import time

    import torch

    P = int(np.prod(lattice))
    rng = np.random.default_rng(seed)
    x = torch.tensor(rng.standard_normal((batch, P, 9)).astype(np.float32), device="cuda")
    y = torch.tensor(rng.standard_normal((batch, P, 3)).astype(np.float32) * 0.1, device="cuda")
    out = {}
    old = os.environ.get("IGAPGPU_NET_TC")
    try:
        for flag in ("1", "0"):
            os.environ["IGAPGPU_NET_TC"] = flag
            net = ConvNet(lattice, batch_max=batch, storage="bf16", params=init_params(seed, zero_last=False))
            o = torch.zeros((batch, P, 3), dtype=torch.float32, device="cuda")
            for _ in range(3):
                net.forward(x, o)
                net.train_step(x, y, 1e-3)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                net.forward(x, o)
            torch.cuda.synchronize()
            tf = (time.perf_counter() - t0) / reps
            t0 = time.perf_counter()
            for _ in range(reps):
                net.train_step(x, y, 1e-3)
            torch.cuda.synchronize()
            tt = (time.perf_counter() - t0) / reps
            out["tensor_cores" if flag == "1" else "scalar"] = {"forward_ms": 1e3 * tf, "train_step_ms": 1e3 * tt}
            net.close()
    finally:
        if old is None:
            os.environ.pop("IGAPGPU_NET_TC", None)
        else:
            os.environ["IGAPGPU_NET_TC"] = old
    return out


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time the predictor's convolutions (tensor cores vs scalar)")
    ap.add_argument("--lattice", default="66,18,18")
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args()
    lat = tuple(int(v) for v in a.lattice.split(","))
    print(json.dumps({"lattice": lat, "batch": a.batch, **time_convolutions(lat, a.batch, a.reps)}))

"""Learned predictor kernels: forward pass and gradients against the FP64
numpy oracle (float storage: 1e-4 relative; bf16 storage: 6e-2, four layers of
BF16 activation rounding over 864-term sums), and a
few Adam steps reduce the loss."""
import numpy as np
import pytest

import conv_oracle as co
import igap4_gb300 as ig
from igap4_gb300.predictor import NPARAM, ConvNet, init_params

pytestmark = pytest.mark.gpu


def _case(seed=0, lattice=(5, 4, 3), B=2):
    rng = np.random.default_rng(seed)
    params = init_params(seed, zero_last=False)
    params[-sum(co.COUT):] = rng.standard_normal(sum(co.COUT)).astype(np.float32) * 0.1
    x = rng.standard_normal((B,) + lattice + (9,)).astype(np.float32)
    y = rng.standard_normal((B,) + lattice + (3,)).astype(np.float32)
    return params, x, y


@pytest.mark.parametrize("storage,tol", [("f32", 1e-4), ("bf16", 6e-2)])
def test_forward_and_gradients_vs_oracle(storage, tol):
    torch = pytest.importorskip("torch")
    lattice, B = (5, 4, 3), 2
    params, x, y = _case(1, lattice, B)
    net = ConvNet(lattice, batch_max=B, storage=storage, params=params)
    P = int(np.prod(lattice))
    xd = torch.tensor(x.reshape(B, P, 9), device="cuda")
    yd = torch.tensor(y.reshape(B, P, 3), device="cuda")
    out = torch.zeros((B, P, 3), dtype=torch.float32, device="cuda")
    net.forward(xd, out)
    loss_ref, grad_ref, y_ref = co.loss_and_grad(params.astype(np.float64), x.astype(np.float64),
                                                 y.astype(np.float64))
    got = out.cpu().numpy().reshape(y_ref.shape)
    assert np.linalg.norm(got - y_ref) <= tol * np.linalg.norm(y_ref)
    loss = net.train_step(xd, yd, 0.0)  # gradients only
    assert abs(loss - loss_ref) <= tol * loss_ref
    g = net.get_grads()
    assert np.linalg.norm(g - grad_ref) <= tol * np.linalg.norm(grad_ref)
    assert g.size == NPARAM


def test_adam_steps_reduce_loss():
    torch = pytest.importorskip("torch")
    lattice, B = (6, 4, 4), 4
    params, x, y = _case(2, lattice, B)
    net = ConvNet(lattice, batch_max=B, storage="bf16", params=params)
    P = int(np.prod(lattice))
    xd = torch.tensor(x.reshape(B, P, 9), device="cuda")
    yd = torch.tensor(y.reshape(B, P, 3), device="cuda") * 0.1
    l0 = net.train_step(xd, yd, 0.0)
    for _ in range(60):
        net.train_step(xd, yd, 3e-3)
    l1 = net.train_step(xd, yd, 0.0)
    assert l1 < 0.5 * l0, (l0, l1)


def test_trained_predictor_reduces_newton_iterations():
    """Small end-to-end run: plain-method trajectories -> training with the
    library's BF16 kernels -> unseen load histories.  The trained predictor
    needs fewer Newton iterations per step than plain Newton from u_n."""
    pytest.importorskip("torch")
    from igap4_gb300 import train_predictor as tp
    from igap4_gb300.predictor import LearnedPredictor

    nelem, dt, amax, steps = (8, 2, 2), 1e-2, 1e-3, 25
    opts = dict(snes_abstol=1e-8, ksp_rtol=1e-5, ksp_restart=60, ksp_max_it=3000, snes_max_it=30, use_graphs=1)
    A, _ = tp.transient_problem(nelem, dt)
    trajs = tp.generate(A, [11, 12, 13], steps, dt, amax, opts)
    X, Y = tp.build_dataset(trajs)
    net, scales, hist = tp.train(A, X, Y, epochs=30, batch=4, lr=2e-3)
    assert hist[-1] < hist[0]
    plain = tp.evaluate(A, [99], steps, dt, amax, None, opts)
    learned = tp.evaluate(A, [99], steps, dt, amax, LearnedPredictor(net, scales), opts)
    print("plain", plain, "learned", learned)
    assert learned["newton_its_per_step"] < plain["newton_its_per_step"]


def test_tensor_core_convolution_matches_scalar(monkeypatch):
    """The 32 -> 32 layers of a BF16 network run as tcgen05 implicit GEMMs
    (forward and data gradient); against the scalar kernels (IGAPGPU_NET_TC=0)
    on a lattice of several 128-point tiles with a partial last tile: the same
    outputs up to BF16 rounding of the differently ordered FP32 sums, and the
    same gradients up to the BF16 rounding of the output gradient."""
    torch = pytest.importorskip("torch")
    lattice, B = (19, 10, 9), 3
    params, x, y = _case(4, lattice, B)
    P = int(np.prod(lattice))
    xd = torch.tensor(x.reshape(B, P, 9), device="cuda")
    yd = torch.tensor(y.reshape(B, P, 3), device="cuda")
    res = {}
    for flag in ("1", "0"):
        monkeypatch.setenv("IGAPGPU_NET_TC", flag)
        net = ConvNet(lattice, batch_max=B, storage="bf16", params=params)
        out = torch.zeros((B, P, 3), dtype=torch.float32, device="cuda")
        n0 = ig.launch_count()
        net.forward(xd, out)
        nl = ig.launch_count() - n0
        loss = net.train_step(xd, yd, 0.0)
        res[flag] = (out.cpu().numpy(), loss, net.get_grads(), nl)
        net.close()
    (o1, l1, g1, n1), (o0, l0, g0, n0) = res["1"], res["0"]
    assert n1 == n0 + 2  # the two 32 -> 32 layers also arrange their weights per tap
    e_out = np.linalg.norm(o1 - o0) / np.linalg.norm(o0)
    e_g = np.linalg.norm(g1 - g0) / np.linalg.norm(g0)
    print(f"tensor-core vs scalar convolution: output {e_out:.2e}, loss {abs(l1 - l0) / l0:.2e}, grads {e_g:.2e}")
    assert e_out <= 2e-2
    assert abs(l1 - l0) <= 2e-2 * l0
    assert e_g <= 3e-2

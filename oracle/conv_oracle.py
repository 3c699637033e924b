"""FP64 numpy oracle of the learned predictor's network (TEST INFRASTRUCTURE).

Same definition as the device kernels: channels-last lattice tensors
[B][nx][ny][nz][C], weights [Co][27][Ci] with tap t = 9(dx+1)+3(dy+1)+(dz+1),
zero padding, ReLU after layers 1-3, mean-square loss.  Used to check the
device forward pass and gradients.
"""
import numpy as np

CIN = (9, 32, 32, 32)
COUT = (32, 32, 32, 3)


def unpack(params):
    Ws, bs = [], []
    off = 0
    for ci, co in zip(CIN, COUT):
        n = co * 27 * ci
        Ws.append(params[off:off + n].reshape(co, 27, ci))
        off += n
    for co in COUT:
        bs.append(params[off:off + co])
        off += co
    return Ws, bs


def _shift(x, t):
    """y[b,i,j,k,:] = x[b,i+dx,j+dy,k+dz,:] with zero padding."""
    dx, dy, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
    B, nx, ny, nz, C = x.shape
    y = np.zeros_like(x)
    xs = slice(max(0, -dx), nx - max(0, dx)), slice(max(0, -dy), ny - max(0, dy)), slice(max(0, -dz), nz - max(0, dz))
    src = slice(max(0, dx), nx + min(0, dx)), slice(max(0, dy), ny + min(0, dy)), slice(max(0, dz), nz + min(0, dz))
    y[:, xs[0], xs[1], xs[2], :] = x[:, src[0], src[1], src[2], :]
    return y


def _unshift(g, t):
    """adjoint of _shift: z[b,p+off,:] += g[b,p,:]"""
    return _shift(g, 26 - t)


def forward(params, x):
    Ws, bs = unpack(params)
    acts = [x]
    pre = []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = np.zeros(x.shape[:4] + (W.shape[0],))
        for t in range(27):
            z += _shift(acts[-1], t) @ W[:, t, :].T
        z += b
        pre.append(z)
        acts.append(np.maximum(z, 0.0) if l < 3 else z)
    return acts, pre


def loss_and_grad(params, x, target):
    Ws, bs = unpack(params)
    acts, pre = forward(params, x)
    y = acts[-1]
    n = y.size
    loss = float(np.mean((y - target) ** 2))
    d = 2.0 * (y - target) / n
    gW = [None] * 4
    gb = [None] * 4
    for l in range(3, -1, -1):
        if l < 3:
            d = d * (pre[l] > 0)
        inp = acts[l]
        W = Ws[l]
        gW[l] = np.zeros_like(W)
        for t in range(27):
            sx = _shift(inp, t)
            gW[l][:, t, :] = np.einsum("bijko,bijkc->oc", d, sx)
        gb[l] = d.sum(axis=(0, 1, 2, 3))
        if l > 0:
            dn = np.zeros(inp.shape)
            for t in range(27):
                dn += _unshift(d @ W[:, t, :], t)
            d = dn
    grad = np.concatenate([g.ravel() for g in gW] + [g.ravel() for g in gb])
    return loss, grad, y

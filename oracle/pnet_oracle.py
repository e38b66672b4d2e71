"""FP64 restatement of the proposal network's forward pass, loss and backward pass (test
infrastructure only: the oracle of the GPU training kernels, never part of the product).

It follows the kernels' arithmetic step by step, including where they round to bf16:
- the GEMM operands: inputs, weights, hidden activations after GELU, and output gradients;
- f32 bias gradients, which the kernels take from the unrounded gradients.
It differs from the kernels only in evaluating everything else in FP64.

The network has no counterpart in the reference. The loss (relaxed winner-take-all L2 over
proposals plus cross-entropy on the proposal logits) is the one the kernels document.
"""
import numpy as np

XY_SCALE = 4.0
EPS_WTA = 0.05


def bf16(a):
    """Round to the nearest bf16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    k = np.sqrt(2.0 / np.pi)
    return 0.5 * z * (1.0 + np.tanh(k * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    k = np.sqrt(2.0 / np.pi)
    t = np.tanh(k * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * k * (1 + 3 * 0.044715 * z * z)


def wrap_pi(a):
    return a - 2 * np.pi * np.floor((a + np.pi) / (2 * np.pi))


def unpack(params, dims):
    """Flat parameter vector (W [out x in] row-major, then b, layer by layer) -> list."""
    out, off = [], 0
    for i, o in zip(dims[:-1], dims[1:]):
        W = params[off:off + i * o].reshape(o, i).astype(np.float64)
        off += i * o
        b = params[off:off + o].astype(np.float64)
        off += o
        out.append((W, b))
    return out


def loss_and_grad_out(O, T, P, yaw_weight=8.0):
    """Mean loss and dL/dO for outputs O [B x 4P] and targets T [B x 3]."""
    B = len(O)
    o = O.reshape(B, P, 4)
    tx, ty, tyaw = T[:, 0] / XY_SCALE, T[:, 1] / XY_SCALE, T[:, 2]
    ex = o[:, :, 0] - tx[:, None]
    ey = o[:, :, 1] - ty[:, None]
    ea = yaw_weight * wrap_pi(np.pi * o[:, :, 2] - tyaw[:, None]) / np.pi
    e = ex ** 2 + ey ** 2 + ea ** 2
    jb = np.argmin(e, axis=1)
    lg = o[:, :, 3]
    mx = lg.max(1, keepdims=True)
    lse = mx[:, 0] + np.log(np.exp(lg - mx).sum(1))
    w_other = EPS_WTA / (P - 1) if P > 1 else 0.0
    best = e[np.arange(B), jb]
    L = best + (lse - lg[np.arange(B), jb]) + w_other * (e.sum(1) - best)
    w = np.full((B, P), w_other)
    w[np.arange(B), jb] = 1.0
    g = np.zeros_like(o)
    g[:, :, 0] = 2 * ex * w / B
    g[:, :, 1] = 2 * ey * w / B
    g[:, :, 2] = 2 * ea * yaw_weight * w / B
    sm = np.exp(lg - lse[:, None])
    sm[np.arange(B), jb] -= 1.0
    g[:, :, 3] = sm / B
    return L.mean(), g.reshape(B, 4 * P)


def forward_backward(params, dims, x, T, P, yaw_weight=8.0):
    """Mean loss and the flat gradient, with the kernels' rounding points."""
    layers = unpack(params, dims)
    X = [bf16(x)]
    Z = []
    for li, (W, b) in enumerate(layers):
        z = X[-1] @ bf16(W).T + b
        Z.append(z)
        if li < len(layers) - 1:
            X.append(bf16(gelu(z)))
    L, dO = loss_and_grad_out(Z[-1], T, P, yaw_weight)
    grads = [None] * len(layers)
    dz = dO
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        dzb = bf16(dz)
        gW = dzb.T @ X[li]
        gb = dz.sum(0)
        grads[li] = (gW, gb)
        if li > 0:
            dx = dzb @ bf16(W)
            dz = dx * gelu_grad(Z[li - 1])
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return L, flat

"""The proposal network's FP64 restatement (oracle/pnet_oracle.py) checked on the CPU: its
loss gradient against central differences, and the full backward pass against central
differences of the loss with bf16 rounding switched off."""
import numpy as np

from oracle import pnet_oracle as O


def test_loss_gradient_finite_differences():
    rng = np.random.default_rng(0)
    P, B = 16, 8
    out = rng.normal(0, 0.5, (B, 4 * P))
    T = np.stack([rng.uniform(-5, 5, B), rng.uniform(-5, 5, B), rng.uniform(-3, 3, B)], 1)
    _, g = O.loss_and_grad_out(out, T, P)
    h = 1e-6
    for _ in range(40):
        i, j = rng.integers(B), rng.integers(4 * P)
        op, om = out.copy(), out.copy()
        op[i, j] += h
        om[i, j] -= h
        num = (O.loss_and_grad_out(op, T, P)[0] - O.loss_and_grad_out(om, T, P)[0]) / (2 * h)
        assert abs(num - g[i, j]) <= 1e-6 + 1e-5 * abs(num)


def test_backward_finite_differences(monkeypatch):
    monkeypatch.setattr(O, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.default_rng(1)
    dims = [8, 6, 6, 64]
    n = sum(i * o + o for i, o in zip(dims[:-1], dims[1:]))
    params = rng.normal(0, 0.4, n)
    x = rng.uniform(0, 1, (5, 8))
    T = np.stack([rng.uniform(-5, 5, 5), rng.uniform(-5, 5, 5), rng.uniform(-3, 3, 5)], 1)
    L, g = O.forward_backward(params, dims, x, T, 16)
    h = 1e-6
    for k in rng.choice(n, 40, replace=False):
        p1, p2 = params.copy(), params.copy()
        p1[k] += h
        p2[k] -= h
        num = (O.forward_backward(p1, dims, x, T, 16)[0] -
               O.forward_backward(p2, dims, x, T, 16)[0]) / (2 * h)
        assert abs(num - g[k]) <= 1e-6 + 1e-4 * abs(num), k


def test_bf16_rounding_ties_to_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], np.float32)
    r = O.bf16(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8

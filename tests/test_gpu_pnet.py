"""The proposal network on the GPU: the tcgen05 GEMM against a torch FP32 matmul, and the
training kernels' loss and gradients against the FP64 restatement (oracle/pnet_oracle.py)."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (256, 512, 576), (64, 512, 256),
                                   (256, 64, 512), (300, 200, 128), (256, 512, 36864)])
def test_gemm_bf16_matches_torch(gpu, m, n, k):
    import torch
    g = torch.Generator(device="cpu").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(n, k, generator=g).to(torch.bfloat16).cuda()
    d = capi.gemm_bf16(a, b)
    ref = a.float() @ b.float().T
    torch.testing.assert_close(d, ref, rtol=1e-3, atol=1e-3 * float(ref.abs().max()))


def test_pnet_gradients_match_fp64_restatement(gpu):
    from oracle import pnet_oracle as O
    cfg = dict(input_dim=128, hidden=64, hidden_layers=2, proposals=16, batch=64, seed=3)
    net = capi.PNet(**cfg)
    dims = [128, 64, 64, 64]
    rng = np.random.default_rng(1)
    x = (rng.uniform(0, 1, (64, 128)) < 0.3).astype(np.float32)
    T = np.stack([rng.uniform(-5, 5, 64), rng.uniform(-5, 5, 64),
                  rng.uniform(-np.pi, np.pi, 64)], 1).astype(np.float32)
    params = net.params()
    loss, g = net.debug_grad(x, T)
    Lr, gr = O.forward_backward(params, dims, x.astype(np.float64), T.astype(np.float64), 16)
    assert abs(loss - Lr) <= 1e-3 * abs(Lr)
    off = 0
    for i, o in zip(dims[:-1], dims[1:]):
        for n in (i * o, o):  # W then b
            a, r = g[off:off + n], gr[off:off + n]
            assert np.linalg.norm(a - r) <= 2e-2 * np.linalg.norm(r) + 1e-7, (off, n)
            off += n
    net.close()


def test_pnet_training_reduces_loss(gpu):
    """A few hundred Adam steps on one synthetic map lower the training loss."""
    from cuda_ndt_matcher_gb300 import synth
    net = capi.PNet(batch=128, seed=5)
    w = synth.search_queries(seed=31, n_queries=24)
    mid = net.add_map(w.map_points)
    for s, t in zip(w.scans, w.true_poses):
        net.add_scan(mid, s, t)
    loss = net.train(300)
    assert np.all(np.isfinite(loss))
    assert loss[-50:].mean() < loss[:20].mean() - 0.3, (loss[:20].mean(), loss[-50:].mean())
    net.close()

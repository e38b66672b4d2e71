"""The proposal network on the GPU: the tcgen05 GEMM against a torch FP32 matmul, and the
training kernels' loss and gradients against the FP64 restatement (oracle/pnet_oracle.py)."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k,splits", [(128, 128, 64, 1), (256, 512, 576, 1),
                                          (64, 512, 256, 1), (256, 64, 512, 1),
                                          (300, 200, 128, 1), (256, 512, 36864, 1),
                                          (256, 512, 36864, 16), (256, 512, 4096, 7)])
def test_gemm_bf16_matches_torch(gpu, m, n, k, splits):
    import torch
    g = torch.Generator(device="cpu").manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(n, k, generator=g).to(torch.bfloat16).cuda()
    d = capi.gemm_bf16(a, b, splits)
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


def _success(pose, truth):
    dyaw = (pose[5] - truth[5] + np.pi) % (2 * np.pi) - np.pi
    return np.linalg.norm(pose[:2] - truth[:2]) < 0.2 and abs(dyaw) < np.radians(1.0)


def test_learned_proposals_gain_over_random_particles(gpu):
    """What the trained network adds. Held-out scans on the training maps, coarse poses off by
    U(+-5 m) in x, y with an unknown heading: with the same budget of 16 NDT refinements per
    query, the network's proposals succeed (error < 0.2 m and < 1 deg) far more often than 16
    random particles drawn over the same range."""
    from cuda_ndt_matcher_gb300 import synth
    maps = synth.proposal_maps(seed=300, n_maps=8, n_train=250, n_test=15)
    net = capi.PNet(seed=11)
    ctx = capi.Context(cuda_graph=1)
    mids = []
    for m in maps:
        mid = net.add_map(m.map_points)
        mids.append(mid)
        ctx.set_target(m.map_points)
        conv = ctx.align_batch(m.train_scans, m.train_poses)
        for s, r in zip(m.train_scans, conv):
            net.add_scan(mid, s, r["pose"])
    net.train(6000)
    rng = np.random.default_rng(5)
    ok_learned = ok_random = n = 0
    for m, mid in zip(maps, mids):
        ctx.set_target(m.map_points)
        coarse = []
        for t in m.test_poses:
            c = t.copy()
            c[:2] += rng.uniform(-5, 5, 2)
            c[5] = rng.uniform(-np.pi, np.pi)
            coarse.append(c)
        learned = ctx.learned_pose_search(net, mid, m.test_scans, coarse)
        # the refinement round keeps the better of its winner and the proposals' winner
        refined = ctx.learned_pose_search(
            net, mid, m.test_scans, coarse,
            refine=dict(num_particles=8, xy_range=0.5, yaw_range=np.radians(5.0), seed=5))
        for a, b in zip(refined, learned):
            assert a["selection_score"] >= b["selection_score"]
        rand = ctx.initial_pose_search(m.test_scans, coarse, num_particles=16, xy_range=5.0,
                                       yaw_range=np.pi, seed=9)
        ok_learned += sum(_success(e["pose"], t) for e, t in zip(learned, m.test_poses))
        ok_random += sum(_success(e["pose"], t) for e, t in zip(rand, m.test_poses))
        n += len(m.test_poses)
    assert ok_learned / n >= ok_random / n + 0.1, (ok_learned / n, ok_random / n)
    net.close()

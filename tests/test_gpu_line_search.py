"""Line search (use_line_search = 1) against the FP64 oracle, through the C ABI. Graph path:
8 candidate steps 0.618^k along the Newton direction, strong Wolfe selection
(src/cuda_ffi/csrc/ndt_graph_kernels.cu:388-430, 473-570, 626-710). CPU path: the
More-Thuente search of NdtOptimizer::align (solver.rs:268-280, 640-700).

Tolerances are those of the clamped-step path (test_gpu_align.py)."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import NdtScanMatcher, capi, matcher, synth
from test_gpu_align import assert_parity

pytestmark = pytest.mark.gpu

LS = dict(ls_candidates=8)


def test_line_search_single_parity(gpu, oracle, single_cases):
    for i, case in enumerate(single_cases):
        ctx = capi.Context(use_line_search=1, cluster_size=4)
        ctx.set_target(case.map_points)
        got = ctx.align(case.scan, case.guess)
        want = oracle.Grid(case.map_points, 2.0).align(case.scan, case.guess, **LS)
        assert_parity(got, want, f"case {i} line search")
        err = np.linalg.norm(got["pose"][:2] - case.true_pose[:2])
        assert got["converged"] and err < 0.1, (i, err)


def test_line_search_stepwise(gpu, oracle, single_cases):
    """One GPU iteration (main pass, candidate pass, Wolfe selection) from every iterate of
    the oracle's line-search trajectory lands on the oracle's next iterate."""
    for case in single_cases:
        g = oracle.Grid(case.map_points, 2.0)
        w, tw = g.align_trace(case.scan, case.guess, **LS)
        starts = tw[:, 3:9]
        nexts = np.vstack([starts[1:], w["pose"][None]])
        ctx = capi.Context(use_line_search=1, max_iterations=1)
        ctx.set_target(case.map_points)
        res = ctx.align_multi_pose(case.scan, list(starts))
        for i, r in enumerate(res):
            dp = np.abs(r["pose"][:3] - nexts[i][:3]).max()
            dr = np.abs(r["pose"][3:] - nexts[i][3:]).max()
            assert dp <= 1e-6 and dr <= 1e-7, ("step", i, dp, dr)


def test_line_search_batch_uneven(gpu, oracle):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=40, scan_points=0)
    rng = np.random.default_rng(2)
    ks = [5, 13, 21, 29]
    scans = []
    for k in ks:
        s = seq.scan(k)
        m = int(rng.integers(2000, min(len(s), 30_000) + 1))
        scans.append(s[np.sort(rng.choice(len(s), m, replace=False))])
    poses = [seq.guess(k) for k in ks]
    g = oracle.Grid(seq.map, 2.0)
    for shape in ((1, 128), (8, 256), (2, 512)):
        ctx = capi.Context(use_line_search=1, cluster_size=shape[0], threads_per_cta=shape[1])
        ctx.set_target(seq.map)
        batch = ctx.align_batch(scans, poses)
        for j, (s, p) in enumerate(zip(scans, poses)):
            assert_parity(batch[j], g.align(s, p, **LS), f"scan {j} shape {shape}")


def test_line_search_graph_replay(gpu):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=40, scan_points=4000)
    scans = [seq.scan(k) for k in (3, 9, 15)]
    poses = [seq.guess(k) for k in (3, 9, 15)]
    direct = capi.Context(use_line_search=1)
    graph = capi.Context(use_line_search=1, cuda_graph=1)
    for c in (direct, graph):
        c.set_target(seq.map)
    for _ in range(2):
        want = direct.align_batch(scans, poses)
        got = graph.align_batch(scans, poses)
        for w, r in zip(want, got):
            np.testing.assert_array_equal(r["pose"], w["pose"])
            assert r["iterations"] == w["iterations"]


def test_matcher_line_search_paths(gpu, single_cases):
    """NdtScanMatcherBuilder::use_line_search: the GPU path runs the parallel line search,
    the CPU path (align_batch) its More-Thuente search."""
    case = single_cases[0]
    m = NdtScanMatcher.builder().resolution(2.0).use_line_search(True).use_gpu(True).build()
    m.set_target(case.map_points)
    r = m.align(case.scan, matcher.pose_vector_to_isometry(case.guess))
    assert r.converged
    rb = m.align_batch(case.scan, [matcher.pose_vector_to_isometry(case.guess)])
    assert rb[0].converged


# ---- CPU path: NdtOptimizer::align with the More-Thuente search (solver.rs:268-280,
# 640-700; more_thuente.rs), one trial pass per search step on the cluster kernel

def _pairs_agree(ctx, tw, index=0):
    """This build's per-iteration correspondence counts equal the oracle's (no point-voxel
    pair at the radius boundary went the other way between the f32 and FP64 tests)."""
    t = ctx.read_trace(index)
    return len(t) == len(tw) and np.array_equal(t[:, 2], tw[:, 2])


def test_cpu_line_search_single_parity(gpu, oracle, single_cases):
    """The seeded scenes: with the search the CPU path converges (the plain one wanders to
    30 iterations on two of them). Where every iteration saw the oracle's pair set, the full
    parity bar; where a boundary pair flipped (the f32 radius test), the search's accept /
    interpolate decisions amplify the difference along the trajectory, so the outcome
    (iterations, convergence, status) and the pose within 1e-3 m."""
    strict = 0
    for i, case in enumerate(single_cases):
        ctx = capi.Context(semantics=capi.SEMANTICS_CPU, use_line_search=1)
        ctx.set_target(case.map_points)
        ctx.trace(True)
        got = ctx.align(case.scan, case.guess)
        want, tw = oracle.Grid(case.map_points, 2.0).align_trace(
            case.scan, case.guess, semantics="cpu", **LS)
        assert want["converged"], i
        if _pairs_agree(ctx, tw):
            assert_parity(got, want, f"case {i} CPU line search")
            strict += 1
        else:
            assert got["iterations"] == want["iterations"], i
            assert got["converged"] and got["status"] == want["status"], i
            assert np.abs(got["pose"][:3] - want["pose"][:3]).max() <= 1e-3, i
            assert np.abs(got["pose"][3:] - want["pose"][3:]).max() <= 1e-4, i
    assert strict >= 2, strict


def test_cpu_line_search_batch_uneven(gpu, oracle):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=40, scan_points=0)
    rng = np.random.default_rng(6)
    ks = [5, 13, 21, 29]
    scans = []
    for k in ks:
        s = seq.scan(k)
        m = int(rng.integers(2000, min(len(s), 30_000) + 1))
        scans.append(s[np.sort(rng.choice(len(s), m, replace=False))])
    poses = [seq.guess(k) for k in ks]
    g = oracle.Grid(seq.map, 2.0)
    want = [g.align(s, p, semantics="cpu", **LS) for s, p in zip(scans, poses)]
    for shape in ((1, 128), (8, 256), (2, 512)):
        ctx = capi.Context(semantics=capi.SEMANTICS_CPU, use_line_search=1,
                           cluster_size=shape[0], threads_per_cta=shape[1])
        ctx.set_target(seq.map)
        batch = ctx.align_batch(scans, poses)
        for j in range(len(scans)):
            if not want[j]["converged"]:  # wandering trajectories: outcome class only
                assert batch[j]["status"] == want[j]["status"]
                continue
            assert_parity(batch[j], want[j], f"scan {j} shape {shape}")


def test_cpu_line_search_stepwise(gpu, oracle, single_cases):
    """One Newton step with the More-Thuente search from every iterate of the oracle's
    trajectory lands on the oracle's next iterate: the search's trials and its accept /
    interpolate decisions match step by step."""
    for c, case in enumerate(single_cases):
        g = oracle.Grid(case.map_points, 2.0)
        _, tw = g.align_trace(case.scan, case.guess, semantics="cpu", **LS)
        starts, nexts = tw[:-1, 3:9], tw[1:, 3:9]
        ctx = capi.Context(semantics=capi.SEMANTICS_CPU, use_line_search=1, max_iterations=2)
        ctx.set_target(case.map_points)
        ctx.trace(True)
        ctx.align_multi_pose(case.scan, list(starts))
        same = 0
        for i in range(len(starts)):
            t = ctx.read_trace(i)
            assert len(t) >= 2, (c, i)
            dp = np.abs(t[1, 3:6] - nexts[i][:3]).max()
            dr = np.abs(t[1, 6:9] - nexts[i][3:]).max()
            if t[0, 2] == tw[i, 2]:  # the oracle's pair set at the start pose
                assert dp <= 1e-6 and dr <= 1e-7, ("step", c, i, dp, dr)
                same += 1
            else:  # a boundary pair flipped: the step moves by its share of the gradient
                assert dp <= 1e-5 and dr <= 1e-5, ("step", c, i, dp, dr)
        assert same >= 0.6 * len(starts), (c, same, len(starts))

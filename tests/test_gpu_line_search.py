"""Graph path with the parallel line search (use_line_search = 1) against the FP64 oracle,
through the C ABI: 8 candidate steps 0.618^k along the Newton direction, strong Wolfe
selection (src/cuda_ffi/csrc/ndt_graph_kernels.cu:388-430, 473-570, 626-710).

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
    """NdtScanMatcherBuilder::use_line_search: the GPU path runs it; the CPU path's
    More-Thuente search is not built and says so."""
    case = single_cases[0]
    m = NdtScanMatcher.builder().resolution(2.0).use_line_search(True).use_gpu(True).build()
    m.set_target(case.map_points)
    r = m.align(case.scan, matcher.pose_vector_to_isometry(case.guess))
    assert r.converged
    with pytest.raises(NotImplementedError):
        m.align_batch(case.scan, [matcher.pose_vector_to_isometry(case.guess)])

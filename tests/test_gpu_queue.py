"""The work-queue Newton kernel (config work_queue = n: a persistent grid claims chunks of n
points per thread of any alignment's iteration; the CTA that completes an iteration runs the
Newton step) against the FP64 oracle and against the cluster kernel, through the C ABI.

Its per-iteration sums are those of the cluster kernel over a different summation tree
(chunk partials summed in chunk order), so each is held to the oracle's tolerances."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth
from parity_helpers import shadow_check, trajectory_has_indefinite_hessian
from test_gpu_align import assert_parity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("semantics", [0, 1])
@pytest.mark.parametrize("threads,ppt", [(256, 4), (128, 1), (512, 2)])
def test_single_alignment_parity_queue(gpu, oracle, single_cases, semantics, threads, ppt):
    sem_name = "gpu" if semantics == 0 else "cpu"
    for i, case in enumerate(single_cases):
        ctx = capi.Context(semantics=semantics, work_queue=ppt, threads_per_cta=threads)
        ctx.set_target(case.map_points)
        got = ctx.align(case.scan, case.guess)
        want = oracle.Grid(case.map_points, 2.0).align(case.scan, case.guess, semantics=sem_name)
        if sem_name == "cpu" and not want["converged"]:
            # clamped-Hessian wandering (newton.rs:118-144): the end point depends on rounding
            assert np.all(np.isfinite(got["pose"])) and got["score"] > 0
            continue
        assert_parity(got, want, f"case {i} {sem_name} queue T={threads} ppt={ppt}")


def test_queue_stepwise(gpu, oracle, single_cases):
    """One iteration (max_iterations = 1) from every oracle iterate lands on the next one;
    the trace the controller records matches the oracle's."""
    for case in single_cases:
        g = oracle.Grid(case.map_points, 2.0)
        w, tw = g.align_trace(case.scan, case.guess)
        starts = tw[:, 3:9]
        nexts = np.vstack([starts[1:], w["pose"][None]])
        ctx = capi.Context(work_queue=1, threads_per_cta=128, max_iterations=1)
        ctx.set_target(case.map_points)
        ctx.trace(True)
        res = ctx.align_multi_pose(case.scan, list(starts))
        for i, r in enumerate(res):
            tg = ctx.read_trace(i)
            assert abs(tg[0, 1] - tw[i, 1]) <= 1e-6 * abs(tw[i, 1]), ("score", i)
            dp = np.abs(r["pose"][:3] - nexts[i][:3]).max()
            dr = np.abs(r["pose"][3:] - nexts[i][3:]).max()
            assert dp <= 1e-6 and dr <= 1e-7, ("step", i, dp, dr)


def test_queue_batch_uneven(gpu, oracle):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=40, scan_points=0)
    rng = np.random.default_rng(1)
    ks = [3, 7, 11, 19, 23, 31]
    scans = []
    for k in ks:
        s = seq.scan(k)
        m = int(rng.integers(2000, min(len(s), 40_000) + 1))
        scans.append(s[np.sort(rng.choice(len(s), m, replace=False))])
    scans.append(scans[0][:600])  # fewer points than one chunk
    ks.append(3)
    poses = [seq.guess(k) for k in ks]
    ctx = capi.Context(work_queue=4)
    ctx.set_target(seq.map)
    batch = ctx.align_batch(scans, poses)
    g = oracle.Grid(seq.map, 2.0)
    for j, (s, p) in enumerate(zip(scans, poses)):
        want = g.align(s, p, semantics="gpu")
        if j == len(scans) - 1:  # 600 points: only the outcome class is compared
            assert batch[j]["status"] == want["status"]
            continue
        assert_parity(batch[j], want, f"batch scan {j} ({len(s)} pts)")


def test_queue_many_alignments(gpu, oracle):
    """More alignments than the grid has CTAs, each from several starts: results identical
    across runs and graph replays; agreement with the oracle no worse than the cluster
    kernel's."""
    seq = synth.Sequence(seed=7, n_map=1_000_000, n_scans=100, scan_points=3000)
    rng = np.random.default_rng(3)
    base = [seq.scan(k) for k in range(100)]
    scans, poses = [], []
    for rep in range(4):
        for k in range(100):
            p = seq.guess(k).copy()
            if rep:
                p[:2] += rng.uniform(-0.3, 0.3, 2)
                p[5] += rng.uniform(-0.02, 0.02)
            scans.append(base[k])
            poses.append(p)
    queue = capi.Context(work_queue=2)
    graph = capi.Context(work_queue=2, cuda_graph=1)
    cluster = capi.Context(work_queue=-1)
    for c in (queue, graph, cluster):
        c.set_target(seq.map)
    a = queue.align_batch(scans, poses)
    b = queue.align_batch(scans, poses)
    g1 = graph.align_batch(scans, poses)
    g2 = graph.align_batch(scans, poses)
    for x, y, z, u in zip(a, b, g1, g2):
        for o in (y, z, u):
            np.testing.assert_array_equal(x["pose"], o["pose"])
            assert x["score"] == o["score"] and x["iterations"] == o["iterations"]
    want = oracle.Grid(seq.map, 2.0).align_batch(scans, poses)
    cl = cluster.align_batch(scans, poses)

    def agree(got):
        return sum(r["iterations"] == w["iterations"] and
                   np.abs(r["pose"][:3] - w["pose"][:3]).max() <= 1e-4 for r, w in zip(got, want))
    # the perturbed starts include trajectories that wander (indefinite Hessians), where two
    # correct summation orders part ways; both kernels are held to the same agreement count
    nq, nc = agree(a), agree(cl)
    assert nq >= 0.8 * len(scans) and nq >= nc - 0.02 * len(scans), (nq, nc)
    # every scan that parts from the oracle: its oracle trajectory crosses an indefinite
    # Hessian, and one GPU iteration from each oracle iterate lands on the next one
    g = oracle.Grid(seq.map, 2.0)
    step = capi.Context(work_queue=2, max_iterations=1)
    step.set_target(seq.map)
    step.trace(True)
    apart = [i for i, (r, w) in enumerate(zip(a, want))
             if not (r["iterations"] == w["iterations"] and
                     np.abs(r["pose"][:3] - w["pose"][:3]).max() <= 1e-4 and
                     np.abs(r["pose"][3:] - w["pose"][3:]).max() <= 1e-5)]
    boundary = 0
    for i in apart:
        assert trajectory_has_indefinite_hessian(g, scans[i], poses[i]), ("definite", i)
        fails, bnd = shadow_check(step, g, scans[i], poses[i])
        assert not fails, ("scan", i, fails)
        boundary += len(bnd)
    assert boundary <= max(4, len(apart)), boundary


def test_queue_autotune_and_forms(gpu):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=16, scan_points=4000)
    import torch
    scans = [seq.scan(k) for k in range(16)]
    xyz = torch.from_numpy(np.concatenate(scans).astype(np.float32)).cuda()
    offsets = np.concatenate([[0], np.cumsum([len(s) for s in scans])]).astype(np.uint64)
    poses = np.stack([seq.guess(k) for k in range(16)])
    for form, allowed in ((1, lambda q: q > 0), (-1, lambda q: q == 0), (0, lambda q: True)):
        ctx = capi.Context(work_queue=form)
        ctx.set_target(seq.map)
        r = ctx.autotune(xyz.data_ptr(), offsets, poses, repeats=1)
        assert allowed(r["work_queue"])
        assert r["candidates"] == {1: 14, -1: 32, 0: 46}[form]
        assert (r["lanes_per_point"] in (1, 2, 4)) == (r["work_queue"] > 0)
        res = ctx.align_batch(scans, list(poses))
        assert all(np.isfinite(x["pose"]).all() for x in res)
    # line search keeps the cluster kernel whatever the form says
    ls = capi.Context(work_queue=4, use_line_search=1)
    ls.set_target(seq.map)
    assert all(x["converged"] for x in ls.align_batch(scans[:4], list(poses[:4])))


def test_queue_streamed_input(gpu):
    """A host batch of more than one copy chunk is copied in while the work-queue kernel runs
    (largest scan first; an alignment's first iteration is claimable once its points are
    resident). Its results are identical to the same batch aligned from device memory (a
    captured graph, replayed), through the synchronous and the asynchronous calls, run to
    run; an empty and a one-point scan ride along."""
    import torch
    seq = synth.Sequence(seed=11, n_map=1_000_000, n_scans=80, scan_points=0)
    rng = np.random.default_rng(5)
    scans, poses = [], []
    for k in range(80):
        s = seq.scan(k)
        m = int(rng.integers(300, min(len(s), 30_000) + 1))
        scans.append(np.ascontiguousarray(s[np.sort(rng.choice(len(s), m, replace=False))]))
        poses.append(seq.guess(k))
    scans[5] = scans[5][:0]
    scans[9] = scans[9][:1]
    assert sum(len(s) for s in scans) * 12 > 4 << 20  # copy chunks of 0.25, 0.5, 1, ... MB
    host = capi.Context(work_queue=2)
    dev = capi.Context(work_queue=2, cuda_graph=1)
    for c in (host, dev):
        c.set_target(seq.map)
    a = host.align_batch(scans, poses)
    b = host.align_batch(scans, poses)
    t = host.batch_submit(scans, poses)
    s1 = host.batch_wait(t)
    xyz = torch.from_numpy(np.concatenate(scans).astype(np.float32)).cuda()
    offsets = np.concatenate([[0], np.cumsum([len(s) for s in scans])]).astype(np.uint64)
    d1 = dev.align_batch_device(xyz.data_ptr(), offsets, poses)
    d2 = dev.align_batch_device(xyz.data_ptr(), offsets, poses)
    for i in range(len(scans)):
        for o in (b, s1, d1, d2):
            np.testing.assert_array_equal(a[i]["pose"], o[i]["pose"])
            np.testing.assert_equal(a[i]["score"], o[i]["score"])
            np.testing.assert_equal(a[i]["nvtl"], o[i]["nvtl"])
            assert a[i]["iterations"] == o[i]["iterations"], i
            assert a[i]["status"] == o[i]["status"], i
    assert sum(r["converged"] for r in a) >= 0.8 * (len(scans) - 2)


_SERIAL_SNIPPET = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from cuda_ndt_matcher_gb300 import capi, synth
seq = synth.Sequence(seed=11, n_map=1_000_000, n_scans=40, scan_points=6000)
scans = [seq.scan(k) for k in range(40)]
poses = [seq.guess(k) for k in range(40)]
ctx = capi.Context(work_queue=2)
ctx.set_target(seq.map)
res = ctx.align_batch(scans, poses)
print(json.dumps([[float(v).hex() for v in r["pose"]] + [r["iterations"]] for r in res]))
"""


def test_queue_streamed_input_serialised(gpu):
    """With every launch synchronous (CUDA_LAUNCH_BLOCKING=1), no copy can run while the
    work-queue kernel waits for input: its CTAs leave after the starvation limit, and the
    continuation launch queued after the last copy finishes the batch. Results are identical
    to those of the concurrent run."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for blocking in ("0", "1"):
        env = dict(os.environ, CUDA_LAUNCH_BLOCKING=blocking)
        r = subprocess.run([sys.executable, "-c", _SERIAL_SNIPPET, root], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[blocking] = json.loads(r.stdout.strip().splitlines()[-1])
    assert sum(len(s) for s in out["0"]) > 0
    assert out["0"] == out["1"]


def test_queue_stall_limit_reports_and_recovers(gpu):
    """The work-queue kernel's no-progress limit runs out without a fault: with every chunk
    of the launch claimed up front (the test hook) no CTA finds work, the call returns
    NDT_ERR_DEVICE with the stall message after the shortened limit, and the next call on the
    same context aligns normally."""
    import time
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=8, scan_points=3000)
    scans = [seq.scan(k) for k in range(8)]
    poses = [seq.guess(k) for k in range(8)]
    ctx = capi.Context(work_queue=2)
    ctx.set_target(seq.map)
    want = ctx.align_batch(scans, poses)
    ctx.debug_queue_stall(1_000_000, withhold_next=True)  # 1 ms
    t0 = time.perf_counter()
    with pytest.raises(capi.NdtError) as e:
        ctx.align_batch(scans, poses)
    assert time.perf_counter() - t0 < 5.0
    assert e.value.code == -8 and "no work for 1 ms" in str(e.value)
    ctx.debug_queue_stall(0)
    got = ctx.align_batch(scans, poses)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a["pose"], b["pose"])
        assert a["iterations"] == b["iterations"]


@pytest.mark.parametrize("lanes", [2, 4])
def test_queue_lanes_per_point(gpu, oracle, single_cases, lanes):
    """Groups of 2 or 4 lanes sharing each point's neighbour search list the same voxels in
    the same order as one lane per point: the batch's results equal the one-lane kernel's
    (same chunks and per-point arithmetic), and single alignments meet the oracle bar."""
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=24, scan_points=0)
    scans = [seq.scan(k) for k in range(0, 24, 2)]
    poses = [seq.guess(k) for k in range(0, 24, 2)]
    one = capi.Context(work_queue=4, threads_per_cta=256, max_registers=64)
    grp = capi.Context(work_queue=4, threads_per_cta=256, max_registers=64,
                       lanes_per_point=lanes)
    for c in (one, grp):
        c.set_target(seq.map)
    a = one.align_batch(scans, poses)
    b = grp.align_batch(scans, poses)
    for x, y in zip(a, b):
        assert x["iterations"] == y["iterations"]
        assert np.abs(x["pose"] - y["pose"]).max() <= 1e-9, np.abs(x["pose"] - y["pose"]).max()
        assert x["num_correspondences"] == y["num_correspondences"]
    for i, case in enumerate(single_cases):
        ctx = capi.Context(work_queue=4, threads_per_cta=256, max_registers=64,
                           lanes_per_point=lanes)
        ctx.set_target(case.map_points)
        got = ctx.align(case.scan, case.guess)
        want = oracle.Grid(case.map_points, 2.0).align(case.scan, case.guess, semantics="gpu")
        assert_parity(got, want, f"case {i} lanes={lanes}")

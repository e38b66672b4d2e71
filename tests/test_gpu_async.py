"""Asynchronous batches (ndt_batch_submit / poll / wait: AsyncBatchPipeline::submit / poll /
wait, src/ndt_cuda/src/optimization/async_pipeline.rs:348-615) through the C ABI."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def seq():
    return synth.Sequence(seed=4, n_map=1_000_000, n_scans=60, scan_points=4000)


def _batches(seq, n_batches, per):
    out = []
    for b in range(n_batches):
        ks = range(2 + b * per, 2 + (b + 1) * per)
        out.append(([seq.scan(k) for k in ks], [seq.guess(k) for k in ks]))
    return out


@pytest.mark.parametrize("form", [-1, 4])
def test_async_batches_match_synchronous(gpu, seq, form):
    """Three batches in flight, collected out of order: each equals ndt_align_batch's
    result for the same scans bit for bit (same kernel, same launch shape)."""
    ctx = capi.Context(work_queue=form)
    ctx.set_target(seq.map)
    batches = _batches(seq, 3, 12)
    want = [ctx.align_batch(s, p) for s, p in batches]
    tickets = [ctx.batch_submit(s, p) for s, p in batches]
    with pytest.raises(capi.NdtError) as e:  # every slot holds a batch
        ctx.batch_submit(*batches[0])
    assert e.value.code == -10
    got = [None] * 3
    for i in (2, 0, 1):
        got[i] = ctx.batch_wait(tickets[i])
    for w, g in zip(want, got):
        for a, b in zip(w, g):
            np.testing.assert_array_equal(a["pose"], b["pose"])
            assert a["score"] == b["score"] and a["nvtl"] == b["nvtl"]
            assert a["iterations"] == b["iterations"]
    with pytest.raises(capi.NdtError):  # a collected ticket is gone
        ctx.batch_wait(tickets[0])


def test_async_poll_and_stream(gpu, seq):
    """A stream of batches with two in flight: poll turns ready, every result arrives, and
    the context's statistics count every alignment."""
    ctx = capi.Context()
    ctx.set_target(seq.map)
    batches = _batches(seq, 4, 8)
    ctx.stats_reset()
    pending, results = [], []
    for s, p in batches:
        if len(pending) == 2:
            results += ctx.batch_wait(pending.pop(0))
        pending.append(ctx.batch_submit(s, p))
    t = pending[-1]
    import time
    t0 = time.time()
    while not ctx.batch_poll(t):
        assert time.time() - t0 < 30
        time.sleep(0.001)
    for t in pending:
        results += ctx.batch_wait(t)
    assert len(results) == 32 and all(r["converged"] for r in results[:8])
    assert ctx.stats()["alignments"] == 32


def test_set_target_drains_batches_in_flight(gpu, seq):
    """A new map while a batch is in flight: the batch finishes on the map it started with
    (its result equals the synchronous one on that map)."""
    ctx = capi.Context()
    ctx.set_target(seq.map)
    scans, poses = _batches(seq, 1, 10)[0]
    want = ctx.align_batch(scans, poses)
    t = ctx.batch_submit(scans, poses)
    ctx.set_target(seq.map[: len(seq.map) // 2])
    got = ctx.batch_wait(t)
    for a, b in zip(want, got):
        np.testing.assert_array_equal(a["pose"], b["pose"])

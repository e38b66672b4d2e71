"""Map tiles streamed in and out with a background rebuild: the map committed from tiles is
bit-identical to set_target on the same points (concatenated in put order); after removing
and adding tiles, an asynchronous commit switches the context to the new map once built,
and alignment then matches a context built directly on the new points."""
import time

import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _quadrants(pts, cx=0.0, cy=0.0):
    return [pts[(pts[:, 0] < cx) & (pts[:, 1] < cy)], pts[(pts[:, 0] >= cx) & (pts[:, 1] < cy)],
            pts[(pts[:, 0] < cx) & (pts[:, 1] >= cy)], pts[(pts[:, 0] >= cx) & (pts[:, 1] >= cy)]]


def _same_map(a, b):
    for x, y in zip(a.map_voxels(), b.map_voxels()):
        assert np.array_equal(x, y)


def test_tiles_commit_and_stream(gpu):
    seq = synth.Sequence(seed=4, n_map=1_000_000, n_scans=40, scan_points=4000)
    tiles = _quadrants(seq.map)
    ctx = capi.Context()
    for i, t in enumerate(tiles):
        ctx.tile_put(i, t)
    ctx.tiles_commit(wait=True)
    ref = capi.Context()
    ref.set_target(np.concatenate(tiles))
    _same_map(ctx, ref)
    st = ctx.tiles_status()
    assert st["tiles"] == 4 and st["points"] == len(seq.map) and not st["pending"]

    # stream: drop the north-east tile, reload it split in two, commit in the background
    ne = tiles[3]
    ctx.tile_remove(3)
    ctx.tile_put(10, ne[: len(ne) // 2])
    ctx.tile_put(11, ne[len(ne) // 2:])
    ctx.tiles_commit(wait=False)
    deadline = time.time() + 30
    while ctx.tiles_status()["pending"] and time.time() < deadline:
        time.sleep(0.001)
    assert ctx.tiles_status()["last_rc"] == 0
    ref2 = capi.Context()
    ref2.set_target(np.concatenate(tiles[:3] + [ne[: len(ne) // 2], ne[len(ne) // 2:]]))
    scans = [seq.scan(k) for k in (5, 9, 13)]
    guesses = [seq.guess(k) for k in (5, 9, 13)]
    got = ctx.align_batch(scans, guesses)   # first call after the rebuild: switches maps
    want = ref2.align_batch(scans, guesses)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g["pose"], w["pose"])
        assert g["nvtl"] == w["nvtl"]
    _same_map(ctx, ref2)
    with pytest.raises(capi.NdtError):
        ctx.tile_remove(3)  # already gone


@pytest.mark.parametrize("res", [2.0, 3.0])
def test_tiles_random_sequence_equals_set_target(gpu, res):
    """Tiles cut at 37 m (not on cell boundaries: cells straddle tiles) put, replaced and
    removed in a seeded random order; after every commit the map equals set_target of the
    resident tiles' points concatenated in put order (a replaced tile keeps its place), bit
    for bit: voxels (cells, means, covariances, inverses, counts), and neighbour lists of
    query points."""
    seq = synth.Sequence(seed=6, n_map=1_000_000, n_scans=4, scan_points=2000)
    pts = seq.map
    tx = np.floor(pts[:, 0] / 37.0).astype(np.int64)
    ty = np.floor(pts[:, 1] / 37.0).astype(np.int64)
    keys = sorted(set(zip(tx.tolist(), ty.tolist())))
    tile_pts = {i: pts[(tx == k[0]) & (ty == k[1])] for i, k in enumerate(keys)}
    rng = np.random.default_rng(12)
    ctx = capi.Context(resolution=res)
    order = []  # resident tile ids in put order
    q = np.concatenate([pts[rng.choice(len(pts), 3000, replace=False)] +
                        rng.normal(0, 0.7, (3000, 3)).astype(np.float32)])
    ids = list(tile_pts)
    tile_pts_now = {}
    for event in range(6):
        for _ in range(int(rng.integers(3, 9))):
            op = rng.random()
            tid = int(rng.choice(ids))
            if op < 0.6 or not order:
                sub = tile_pts[tid]
                if rng.random() < 0.3:  # a replaced tile with fewer points
                    sub = sub[rng.random(len(sub)) < 0.7]
                ctx.tile_put(tid, sub)
                if tid not in order:
                    order.append(tid)
                tile_pts_now[tid] = sub
            else:
                tid = int(rng.choice(order))
                ctx.tile_remove(tid)
                order.remove(tid)
        if not order:
            continue
        ctx.tiles_commit(wait=bool(event % 2))
        ref = capi.Context(resolution=res)
        ref.set_target(np.concatenate([tile_pts_now[t] for t in order]))
        ctx.map_info()  # switches to the merged map once it is ready
        while ctx.tiles_status()["pending"]:
            time.sleep(0.0005)
        ctx.map_info()
        assert ctx.tiles_status()["last_rc"] == 0
        _same_map(ctx, ref)
        for max_nb in (8, 27):
            a = ctx.neighbors(q, max_nb)
            b = ref.neighbors(q, max_nb)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        ref.close()
    ctx.close()

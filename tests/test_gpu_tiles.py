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

"""Large-map voxel build (the 2 x 2 km stress workload, here with 5M points) at 1 m (the
cell box exceeds the dense-index budget: hash lookups) and 2 m (dense index): sampled voxels
bit-exact against the oracle's build of exactly those cells' points, presence of a voxel
exactly where a cell holds enough points, and alignment of dense crop scans."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big_map():
    return synth.large_map(seed=7, extent=2000.0, n_points=5_000_000)


def _cells(pts, res):
    return np.floor(pts / np.float32(res)).astype(np.int64)


@pytest.mark.parametrize("res", [1.0, 2.0])
def test_large_map_sampled_voxels_bitexact(gpu, oracle, big_map, res):
    ctx = capi.Context(resolution=res)
    ctx.set_target(big_map)
    info = ctx.map_info()
    assert (info.dense_grid_mib > 0) == (res == 2.0)
    coords, means, covs, icovs, counts = ctx.map_voxels()
    cells = _cells(big_map, res)
    key = ((cells[:, 0] + (1 << 20)) << 42) | ((cells[:, 1] + (1 << 20)) << 21) | (cells[:, 2] + (1 << 20))
    uk, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
    # a voxel exactly where a cell holds >= 6 points (all such cells regularise here)
    vkey = ((coords[:, 0].astype(np.int64) + (1 << 20)) << 42) | \
           ((coords[:, 1].astype(np.int64) + (1 << 20)) << 21) | (coords[:, 2].astype(np.int64) + (1 << 20))
    assert np.array_equal(np.sort(vkey), uk[cnt >= 6])
    assert counts.sum() == cnt[cnt >= 6].sum()
    rng = np.random.default_rng(int(res * 10))
    pick = rng.choice(len(coords), 60, replace=False)
    order = np.argsort(inv, kind="stable")
    starts = np.concatenate([[0], np.cumsum(cnt)])
    pos = np.searchsorted(uk, vkey[pick])
    for v, u in zip(pick, pos):
        members = np.sort(order[starts[u]:starts[u + 1]])  # the cell's points, input order
        g = oracle.Grid(big_map[members], res, centered=True)
        assert g.n == 1
        assert np.array_equal(g.coords[0], coords[v]) and g.counts[0] == counts[v]
        assert np.array_equal(g.means[0], means[v])
        assert np.array_equal(g.covs[0], covs[v]) and np.array_equal(g.icovs[0], icovs[v])


def test_large_map_dense_scan_alignment(gpu, big_map):
    ctx = capi.Context(resolution=2.0)
    ctx.set_target(big_map)
    rng = np.random.default_rng(3)
    poses, scans, guesses = [], [], []
    for i in range(8):
        p = np.array([rng.uniform(-800, 800), rng.uniform(-800, 800), 1.8, 0, 0,
                      rng.uniform(-np.pi, np.pi)])
        s = synth.crop_scan(big_map, p, 100_000, seed=i)
        g = p.copy()
        g[:2] += rng.uniform(-0.3, 0.3, 2)
        g[5] += np.radians(rng.uniform(-1.0, 1.0))
        poses.append(p)
        scans.append(s)
        guesses.append(g)
    res = ctx.align_batch(scans, guesses)
    err = [np.linalg.norm(r["pose"][:2] - p[:2]) for r, p in zip(res, poses)]
    assert np.median(err) < 0.1, err

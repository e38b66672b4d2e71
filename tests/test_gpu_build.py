"""GPU voxel-map build vs the oracle, through the C ABI: Morton codes, radix sort order,
segments, voxel membership/counts/means bit-exact; covariances / inverse covariances within
2 / 4 f32 ULP of the oracle's centred FP64 restatement and within 1e-4 relative of the
reference's uncentred formula."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth
from parity_helpers import matrix_ulps

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "reference_known_answers.json")))


def _torch():
    import torch
    return torch


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def gpu_sort(keys, vals, begin=0, end=64):
    torch = _torch()
    L = capi.load()
    n = len(keys)
    k = torch.from_numpy(np.asarray(keys, np.uint64).view(np.int64).copy()).cuda()
    v = torch.from_numpy(np.asarray(vals, np.uint32).view(np.int32).copy()).cuda()
    tb = C.c_uint64(0)
    capi.check(L.ndt_radix_sort_pairs_u64_u32(_ptr(k), _ptr(v), n, begin, end, None,
                                              C.byref(tb), None))
    tmp = torch.empty(max(int(tb.value), 1), dtype=torch.uint8, device="cuda")
    capi.check(L.ndt_radix_sort_pairs_u64_u32(_ptr(k), _ptr(v), n, begin, end, _ptr(tmp),
                                              C.byref(tb), None))
    torch.cuda.synchronize()
    return k.cpu().numpy().view(np.uint64), v.cpu().numpy().view(np.uint32)


def gpu_segments(codes):
    torch = _torch()
    L = capi.load()
    n = len(codes)
    k = torch.from_numpy(np.asarray(codes, np.uint64).view(np.int64).copy()).cuda() if n else \
        torch.empty(1, dtype=torch.int64, device="cuda")
    ids = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    starts = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    num = torch.zeros(1, dtype=torch.int32, device="cuda")
    tb = C.c_uint64(0)
    capi.check(L.ndt_detect_segments(_ptr(k), n, _ptr(ids), _ptr(starts), _ptr(num), None,
                                     C.byref(tb), None))
    tmp = torch.empty(max(int(tb.value), 1), dtype=torch.uint8, device="cuda")
    capi.check(L.ndt_detect_segments(_ptr(k), n, _ptr(ids), _ptr(starts), _ptr(num),
                                     _ptr(tmp), C.byref(tb), None))
    torch.cuda.synchronize()
    m = int(num.item())
    return ids.cpu().numpy()[:n], starts.cpu().numpy()[:m], m


def test_radix_sort_golden(gpu):
    g = GOLD["radix_sort"]
    k, v = gpu_sort(g["keys"], g["values"])
    assert list(k) == g["sorted_keys"] and list(v) == g["sorted_values"]
    k, v = gpu_sort(g["stable_keys"], g["stable_values"])
    assert list(v) == g["stable_values"]


@pytest.mark.parametrize("n", [1, 2, 255, 4096, 4097, 100_003, 1_000_000])
def test_radix_sort_bitexact(gpu, oracle, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 64 - 1, n, dtype=np.uint64)
    keys[::5] = keys[0]
    vals = rng.integers(0, 2 ** 32 - 1, n, dtype=np.uint32)
    k, v = gpu_sort(keys, vals)
    ok, ov = oracle.radix_sort_pairs(keys, vals)
    assert np.array_equal(k, ok) and np.array_equal(v, ov)


def test_radix_sort_partial_bits(gpu):
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 2 ** 40, 50_000, dtype=np.uint64)
    vals = np.arange(50_000, dtype=np.uint32)
    k, v = gpu_sort(keys, vals, 4, 27)
    masked = (keys >> np.uint64(4)) & np.uint64((1 << 23) - 1)
    order = np.argsort(masked, kind="stable")
    assert np.array_equal(v, vals[order]) and np.array_equal(k, keys[order])


def test_segments_golden(gpu):
    for case in GOLD["segments"]:
        ids, starts, m = gpu_segments(np.array(case["codes"], np.uint64))
        assert m == case["num"]
        if "ids" in case:
            assert list(ids) == case["ids"]
        if "starts" in case:
            assert list(starts) == case["starts"]


def test_segments_random_bitexact(gpu, oracle):
    rng = np.random.default_rng(3)
    codes = np.sort(rng.integers(0, 5000, 300_000).astype(np.uint64))
    ids, starts, m = gpu_segments(codes)
    oid, ost, on = oracle.detect_segments(codes)
    assert m == on and np.array_equal(ids, oid) and np.array_equal(starts, ost)


def test_morton_codes_bitexact(gpu, oracle):
    torch = _torch()
    L = capi.load()
    case = synth.single_case(1)
    pts = case.map_points.copy()
    pts[::997] = np.nan
    pts[5] = [-17.3, 4.0, -2.0]
    n = len(pts)
    d = torch.from_numpy(pts).cuda()
    codes = torch.empty(n, dtype=torch.int64, device="cuda")
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    mn = torch.empty(3, dtype=torch.int32, device="cuda")
    tb = C.c_uint64(0)
    capi.check(L.ndt_morton_codes(_ptr(d), n, 2.0, _ptr(codes), _ptr(idx), _ptr(mn), None,
                                  C.byref(tb), None))
    tmp = torch.empty(int(tb.value), dtype=torch.uint8, device="cuda")
    capi.check(L.ndt_morton_codes(_ptr(d), n, 2.0, _ptr(codes), _ptr(idx), _ptr(mn), _ptr(tmp),
                                  C.byref(tb), None))
    torch.cuda.synchronize()
    oc, omin, ok = oracle.morton_codes_coord(pts, 2.0)
    assert ok
    assert np.array_equal(codes.cpu().numpy().view(np.uint64), oc)
    assert np.array_equal(mn.cpu().numpy(), omin)
    assert np.array_equal(idx.cpu().numpy(), np.arange(n, dtype=np.int32))


def _ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def _maps():
    c1 = synth.single_case(1)
    hc = synth.half_cubic_pcd() + np.array([100, 100, 0], np.float32)
    seq = synth.Sequence(seed=2, n_map=1_000_000, n_scans=10)
    return {"single": c1.map_points, "half_cube": hc, "sequence_1M": seq.map}


@pytest.mark.parametrize("name", ["single", "half_cube", "sequence_1M"])
def test_map_build_matches_oracle(gpu, oracle, name):
    pts = _maps()[name]
    ctx = capi.Context()
    ctx.set_target(pts)
    coords, means, covs, icovs, counts = ctx.map_voxels()
    g = oracle.Grid(pts, 2.0, centered=True)
    assert len(coords) == g.n
    assert np.array_equal(coords, g.coords)            # membership and Morton order
    assert np.array_equal(counts, g.counts)            # per-voxel counts
    assert np.array_equal(means, g.means)              # FP64 sums in input order
    # regularised covariance and inverse: the library forms them in FP64 from f32 eigenvector
    # directions (Rayleigh quotients, rank-one clamp, adjugate inverse), the oracle from an
    # FP64 Jacobi; both are FP64-accurate, so they agree to f32 rounding
    cu, iu = matrix_ulps(covs, g.covs), matrix_ulps(icovs, g.icovs)
    print(f"{name}: {len(coords)} voxels, covariance max {cu.max():.1f} f32 ULP "
          f"({(cu > 0).sum()} differ), inverse max {iu.max():.1f} f32 ULP ({(iu > 0).sum()} "
          f"differ)")
    assert cu.max() <= 2 and iu.max() <= 4, (cu.max(), iu.max())
    # the reference's uncentred FP64 formula differs only in the last f32 bits
    r = oracle.Grid(pts, 2.0, centered=False)
    assert np.array_equal(coords, r.coords) and np.array_equal(counts, r.counts)
    rel = np.abs(icovs - r.icovs).max() / np.abs(r.icovs).max()
    assert rel < 1e-4, rel
    info = ctx.map_info()
    assert info.num_voxels == g.n and info.hash_capacity == g.capacity


def _route_map():
    """Voxels that take every route of the statistics kernel: cells far from the origin (exact
    sums), cells next to zero with values over many binades, +-0 and subnormals (exact
    covariance, FP64 running sum for the mean), one warp-summed voxel of 3,000 points, one of
    70,000 (beyond the exact sums' bound: FP64 two-pass), and many small ones."""
    rng = np.random.default_rng(5)
    parts = []
    far = np.column_stack([rng.integers(-800, 800, (300, 2)), rng.integers(-40, 40, 300)])
    for c in far:                                       # far cells, 6-60 points
        n = int(rng.integers(6, 60))
        parts.append(c * 2.0 + rng.uniform(0, 2, (n, 3)))
    for _ in range(200):                                # next to zero on z, ground-like
        n = int(rng.integers(6, 40))
        xy = rng.integers(-50, 50, 2) * 2.0 + rng.uniform(0, 2, (n, 2))
        z = rng.normal(0, 0.03, n) * 10.0 ** rng.integers(-6, 1, n)
        parts.append(np.column_stack([xy, z]))
    tiny = np.zeros((12, 3))
    tiny[:, :2] = [10.5, 20.5]
    tiny[:, 2] = [0.0, -0.0, 1e-40, -1e-41, 1e-38, 3e-39, 1e-30, 1e-20, 0.5, 1.5, 1e-7, 0.25]
    parts.append(tiny)                                  # zeros and subnormals
    parts.append(np.array([300.0, 300.0, 4.0]) + rng.uniform(0, 2, (3000, 3)))
    parts.append(np.array([-300.0, 100.0, 6.0]) + rng.uniform(0, 2, (70000, 3)))
    pts = np.concatenate(parts).astype(np.float32)
    return np.ascontiguousarray(pts[rng.permutation(len(pts))])


def test_voxel_routes_match_oracle(gpu, oracle):
    pts = _route_map()
    ctx = capi.Context()
    ctx.set_target(pts)
    coords, means, covs, icovs, counts = ctx.map_voxels()
    g = oracle.Grid(pts, 2.0, centered=True)
    assert np.array_equal(coords, g.coords) and np.array_equal(counts, g.counts)
    assert np.array_equal(means, g.means)
    assert counts.max() == 70000 and (counts == 3000).any()
    cu, iu = matrix_ulps(covs, g.covs), matrix_ulps(icovs, g.icovs)
    print(f"routes: {len(coords)} voxels, covariance max {cu.max():.1f} f32 ULP, inverse max "
          f"{iu.max():.1f} f32 ULP")
    assert cu.max() <= 2 and iu.max() <= 4, (cu.max(), iu.max())


@pytest.mark.parametrize("cell_index", [0, 1])   # dense cell index / hash probing
def test_neighbors_bitexact(gpu, oracle, cell_index):
    case = synth.single_case(2)
    ctx = capi.Context(cell_index=cell_index)
    ctx.set_target(case.map_points)
    assert (ctx.map_info().dense_grid_mib > 0) == (cell_index == 0)
    g = oracle.Grid(case.map_points, 2.0)
    rng = np.random.default_rng(0)
    q = np.concatenate([g.means + rng.normal(0, 0.8, g.means.shape).astype(np.float32),
                        rng.uniform(-60, 60, (5000, 3)).astype(np.float32)])
    for max_nb in (8, 27):
        idx, cnt = ctx.neighbors(q, max_nb)
        oidx, ocnt = g.query_gpu_sem(q, max_nb)
        assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)


def test_build_errors_and_nan(gpu):
    ctx = capi.Context()
    with pytest.raises(capi.NdtError) as e:
        ctx.set_target(np.zeros((0, 3), np.float32))
    assert e.value.code == -3
    with pytest.raises(capi.NdtError) as e:
        ctx.set_target(np.full((100, 3), np.nan, np.float32))
    assert e.value.code == -3
    with pytest.raises(capi.NdtError) as e:  # every voxel below min points
        ctx.set_target(np.random.default_rng(0).uniform(0, 100, (100, 3)).astype(np.float32))
    assert e.value.code == -4
    with pytest.raises(capi.NdtError) as e:
        capi.Context().align(np.zeros((10, 3), np.float32), np.zeros(6))
    assert e.value.code == -2
    case = synth.single_case(1)
    pts = case.map_points.copy()
    ctx.set_target(pts)
    ref = ctx.map_voxels()
    bad = np.concatenate([pts, np.full((50, 3), np.inf, np.float32)])
    ctx.set_target(bad)
    got = ctx.map_voxels()
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)

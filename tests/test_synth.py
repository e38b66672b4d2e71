"""The seeded workload generator is deterministic and has the workload shapes."""
import numpy as np

from cuda_ndt_matcher_gb300 import synth


def test_single_case_deterministic():
    a = synth.single_case(5)
    b = synth.single_case(5)
    assert np.array_equal(a.map_points, b.map_points) and np.array_equal(a.scan, b.scan)
    assert a.map_points.shape == (200_000, 3)
    assert 500 < len(a.scan) < 5000
    assert np.all(np.abs(a.guess[:2] - a.true_pose[:2]) <= 0.5)
    assert abs(np.degrees(a.guess[5] - a.true_pose[5])) <= 2.0


def test_sequence_shapes_small():
    s = synth.Sequence(seed=3, n_map=200_000, n_scans=50)
    assert s.map.shape == (200_000, 3)
    sc = s.scan(10)
    assert sc.shape == (20_000, 3)
    assert np.array_equal(sc, s.scan(10))
    g = s.guess(10)
    assert np.linalg.norm(g[:2] - s.true_pose(10)[:2]) < 1.0


def test_half_cube_and_voxelize():
    p = synth.half_cubic_pcd()
    assert p.shape == (30603, 3)
    v = synth.voxelize_pcd(p, 1.0)
    assert 1000 < len(v) < len(p)
    assert np.all(np.isfinite(v))

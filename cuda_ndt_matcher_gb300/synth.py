"""Seeded synthetic NDT workloads (maps, trajectories, ray-cast lidar scans).

Stands in for the reference's rosbag/PCD data, which is not available. Shapes follow the
benchmark workloads:

- ``single``   : 200k-point map over 100x100 m (12 box buildings, 40 poles), one 32-ring
                 scan downsampled at 1 m, initial guess perturbed by U(+-0.5 m) xy and
                 U(+-2 deg) yaw.
- ``sequence`` : 5M-point map over 400x400 m (250 buildings, 800 poles, 300 tree blobs),
                 a 1000-pose cubic-spline trajectory at 10 m/s and 10 Hz, 128-ring scans
                 downsampled at 0.6 m and subsampled to 20k points; initial guesses = constant-velocity prediction from the
                 previous true poses + N(0, 0.1 m) xy and N(0, 0.5 deg) yaw noise.
"""
import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_synth())
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        L.synth_scene_create.restype = C.c_void_p
        L.synth_scene_create.argtypes = [C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_int,
                                         C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_void_p, C.c_int]
        L.synth_scene_free.argtypes = [C.c_void_p]
        L.synth_scene_counts.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.int32)]
        L.synth_map_points.argtypes = [C.c_void_p, C.c_uint64, C.c_size_t, f32p]
        L.synth_scan.restype = C.c_size_t
        L.synth_scan.argtypes = [C.c_void_p, f64p, C.c_int, C.c_double, C.c_double,
                                 C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_uint64, f32p, C.c_size_t]
        L.synth_trajectory.argtypes = [C.c_uint64, C.c_double, C.c_double, C.c_int,
                                       C.c_double, C.c_double, f64p]
        _lib = L
    return _lib


@dataclass
class Lidar:
    rings: int = 32
    vfov_lo: float = -25.0
    vfov_hi: float = 15.0
    az_step: float = 0.2
    max_range: float = 80.0
    range_sigma: float = 0.02
    leaf: float = 1.0
    dense: int = 0          # rings packed into [band_lo, band_hi]; 0 = uniform spacing
    band_lo: float = -6.0
    band_hi: float = 2.0


class Scene:
    def __init__(self, seed, extent, n_boxes, n_poles, n_trees, clear_xy=None,
                 box_side=(8.0, 30.0), box_h=(5.0, 20.0)):
        clear = None
        nclear = 0
        self._clear = None
        if clear_xy is not None and len(clear_xy):
            self._clear = np.ascontiguousarray(np.asarray(clear_xy, np.float64).reshape(-1, 2))
            clear = self._clear.ctypes.data
            nclear = len(self._clear)
        self.h = lib().synth_scene_create(seed, extent, n_boxes, n_poles, n_trees,
                                          box_side[0], box_side[1], box_h[0], box_h[1],
                                          clear, nclear)
        self.extent = extent
        self.seed = seed
        cnt = np.zeros(3, np.int32)
        lib().synth_scene_counts(self.h, cnt)
        self.counts = tuple(int(c) for c in cnt)

    def __del__(self):
        if getattr(self, "h", None):
            lib().synth_scene_free(self.h)
            self.h = None

    def map_points(self, n, seed=None):
        out = np.zeros((n, 3), np.float32)
        lib().synth_map_points(self.h, self.seed if seed is None else seed, n, out)
        return out

    def scan(self, sensor_pose4, lidar: Lidar, seed):
        """Ray-cast scan in the sensor frame; sensor_pose4 = [x, y, z, yaw]."""
        naz = int(round(360.0 / lidar.az_step))
        cap = naz * lidar.rings
        out = np.zeros((cap, 3), np.float32)
        m = lib().synth_scan(self.h, np.ascontiguousarray(sensor_pose4, np.float64),
                             lidar.rings, lidar.vfov_lo, lidar.vfov_hi, lidar.dense,
                             lidar.band_lo, lidar.band_hi, lidar.az_step,
                             lidar.max_range, lidar.range_sigma, lidar.leaf, seed, out, cap)
        return out[:m].copy()


def trajectory(seed, extent, n, spacing, height=1.8, margin=40.0):
    out = np.zeros((n, 4), np.float64)
    lib().synth_trajectory(seed, extent, margin, n, spacing, height, out)
    return out


def pose6(p4):
    """[x, y, z, yaw] -> pose vector [x, y, z, roll, pitch, yaw]."""
    return np.array([p4[0], p4[1], p4[2], 0.0, 0.0, p4[3]], np.float64)


@dataclass
class SingleCase:
    map_points: np.ndarray
    scan: np.ndarray
    true_pose: np.ndarray
    guess: np.ndarray
    scene: Scene = field(repr=False, default=None)


def single_case(seed=1, n_map=200_000, rings=32):
    """The CPU-runnable single-alignment workload (100x100 m, 200k-point map)."""
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(-25, 25, size=2)
    yaw = rng.uniform(-math.pi, math.pi)
    scene = Scene(seed, 100.0, 12, 40, 0, clear_xy=[[sx, sy]])
    mp = scene.map_points(n_map)
    true4 = np.array([sx, sy, 1.8, yaw])
    scan = scene.scan(true4, Lidar(rings=rings), seed + 1000)
    true6 = pose6(true4)
    guess = true6.copy()
    guess[0] += rng.uniform(-0.5, 0.5)
    guess[1] += rng.uniform(-0.5, 0.5)
    guess[5] += math.radians(rng.uniform(-2.0, 2.0))
    return SingleCase(mp, scan, true6, guess, scene)


class Sequence:
    """The full-scale workload: 400x400 m map, spline trajectory, 128-ring scans."""

    def __init__(self, seed=2, n_map=5_000_000, n_scans=1000, extent=400.0, rings=128,
                 n_boxes=250, n_poles=800, n_trees=300, speed=10.0, rate=10.0,
                 scan_points=20_000):
        self.seed = seed
        self.traj = trajectory(seed, extent, n_scans, speed / rate)
        clear = self.traj[:, :2][::2]
        self.scene = Scene(seed, extent, n_boxes, n_poles, n_trees, clear_xy=clear)
        self.map = self.scene.map_points(n_map)
        self.lidar = Lidar(rings=rings, dense=96, leaf=0.6)
        self.n_scans = n_scans
        self.scan_points = scan_points

    def scan(self, k):
        """Ray-cast scan k, downsampled (0.6 m leaf) and subsampled to `scan_points`.

        With this scene a 1.0 m leaf leaves ~10k points per 128-ring scan; the workload is
        specified per 20k-point scan, so the leaf is 0.6 m (~28k points) followed by a
        seeded uniform subsample to exactly `scan_points` points."""
        pts = self.scene.scan(self.traj[k], self.lidar, self.seed * 100003 + k)
        if self.scan_points and len(pts) > self.scan_points:
            rng = np.random.default_rng([self.seed, 7, k])
            sel = np.sort(rng.choice(len(pts), self.scan_points, replace=False))
            pts = np.ascontiguousarray(pts[sel])
        return pts

    def true_pose(self, k):
        return pose6(self.traj[k])

    def guess(self, k):
        """Constant-velocity prediction from the two previous true poses plus noise."""
        rng = np.random.default_rng([self.seed, k])
        p1 = self.traj[max(k - 1, 0)]
        p2 = self.traj[max(k - 2, 0)]
        pred = p1 + (p1 - p2)
        dyaw = math.atan2(math.sin(p1[3] - p2[3]), math.cos(p1[3] - p2[3]))
        pred[3] = p1[3] + dyaw
        g = pose6(pred)
        g[0] += rng.normal(0, 0.1)
        g[1] += rng.normal(0, 0.1)
        g[5] += math.radians(rng.normal(0, 0.5))
        return g


def half_cubic_pcd(length=20.0, interval=0.2):
    """make_half_cubic_pcd (src/ndt_cuda/src/test_utils.rs:19-45): three orthogonal planes."""
    n = int(np.float32(length) / np.float32(interval)) + 1
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    u = (np.float32(interval) * j.astype(np.float32)).ravel()
    v = (np.float32(interval) * i.astype(np.float32)).ravel()
    z = np.zeros_like(u)
    pts = np.stack([np.stack([u, v, z], 1), np.stack([z, u, v], 1), np.stack([u, z, v], 1)], 1)
    return np.ascontiguousarray(pts.reshape(-1, 3).astype(np.float32))


def voxelize_pcd(points, leaf):
    """voxelize_pcd (src/ndt_cuda/src/test_utils.rs:76-110): centroid per floor(p/leaf) cell,
    FP64 sums, f32 output; cells in ascending key order (the reference's order is a HashMap's)."""
    p = np.asarray(points, np.float32)
    p = p[np.isfinite(p).all(1)]
    inv = np.float32(1.0) / np.float32(leaf)
    cells = np.floor(p * inv).astype(np.int64)
    key = ((cells[:, 0] + (1 << 20)) << 42) | ((cells[:, 1] + (1 << 20)) << 21) | (cells[:, 2] + (1 << 20))
    uk, inv_idx = np.unique(key, return_inverse=True)
    sums = np.zeros((len(uk), 3))
    np.add.at(sums, inv_idx, p.astype(np.float64))
    cnt = np.bincount(inv_idx, minlength=len(uk)).astype(np.float64)
    return np.ascontiguousarray((sums / cnt[:, None]).astype(np.float32))


@dataclass
class SearchWorkload:
    map_points: np.ndarray
    scans: list
    true_poses: np.ndarray
    priors: np.ndarray


def search_queries(seed=21, n_queries=16, n_map=200_000, prior_xy=1.0):
    """Initial-pose queries on one 100x100 m single-workload map: 32-ring scans from seeded
    poses; each prior is the true pose with x, y + U(+-prior_xy) and an unknown heading
    (yaw uniform on the circle)."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-30, 30, size=(n_queries, 2))
    yaw = rng.uniform(-math.pi, math.pi, size=n_queries)
    scene = Scene(seed, 100.0, 12, 40, 0, clear_xy=xy)
    mp = scene.map_points(n_map)
    scans, truth, priors = [], [], []
    for i in range(n_queries):
        t4 = np.array([xy[i, 0], xy[i, 1], 1.8, yaw[i]])
        scans.append(scene.scan(t4, Lidar(rings=32), seed * 100 + i))
        t6 = pose6(t4)
        p = t6.copy()
        p[:2] += rng.uniform(-prior_xy, prior_xy, 2)
        p[5] = rng.uniform(-math.pi, math.pi)
        truth.append(t6)
        priors.append(p)
    return SearchWorkload(mp, scans, np.array(truth), np.array(priors))


@dataclass
class ProposalMap:
    map_points: np.ndarray
    train_scans: list
    train_poses: np.ndarray
    test_scans: list
    test_poses: np.ndarray


def _proposal_map(seed, n_train, n_test, extent, n_map):
    rng = np.random.default_rng(seed)
    n = n_train + n_test
    xy = rng.uniform(-extent / 2 + 30, extent / 2 - 30, size=(n, 2))
    yaw = rng.uniform(-math.pi, math.pi, size=n)
    area = (extent / 400.0) ** 2  # sequence-workload densities per area
    scene = Scene(seed, extent, int(250 * area), int(800 * area), int(300 * area), clear_xy=xy)
    mp = scene.map_points(n_map)
    scans, poses = [], []
    for i in range(n):
        t4 = np.array([xy[i, 0], xy[i, 1], 1.8, yaw[i]])
        scans.append(scene.scan(t4, Lidar(rings=32), seed * 1000 + i))
        poses.append(pose6(t4))
    poses = np.array(poses)
    return ProposalMap(mp, scans[:n_train], poses[:n_train], scans[n_train:], poses[n_train:])


def proposal_maps(seed=100, n_maps=16, n_train=400, n_test=25, extent=200.0,
                  n_map=1_250_000, threads=None):
    """Maps for the learned initial-pose proposals: 200x200 m tiles of the sequence-workload
    generator (same densities of buildings, poles and tree blobs), each with 32-ring scans
    from seeded poses split into training and held-out test scans. The ray casts run in C
    (outside the GIL), so maps are generated in parallel threads."""
    from concurrent.futures import ThreadPoolExecutor
    threads = threads or min(n_maps, os.cpu_count() or 1)
    with ThreadPoolExecutor(threads) as ex:
        return list(ex.map(lambda m: _proposal_map(seed + m, n_train, n_test, extent, n_map),
                           range(n_maps)))


def queue_scans(seed=22, n_scans=64, lo=2000, hi=40000, n_map=200_000):
    """A queue of scans of uneven size on one single-workload map: 128-ring scans (dense
    band) from seeded poses, each subsampled to a log-uniform size in [lo, hi] (capped by
    what the ray cast returns); guesses perturbed like the single workload."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-30, 30, size=(n_scans, 2))
    yaw = rng.uniform(-math.pi, math.pi, size=n_scans)
    scene = Scene(seed, 100.0, 12, 40, 0, clear_xy=xy)
    mp = scene.map_points(n_map)
    lidar = Lidar(rings=128, dense=96, leaf=0.3)
    scans, truth, guesses = [], [], []
    for i in range(n_scans):
        t4 = np.array([xy[i, 0], xy[i, 1], 1.8, yaw[i]])
        s = scene.scan(t4, lidar, seed * 100 + i)
        m = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        m = min(m, len(s))
        scans.append(np.ascontiguousarray(s[np.sort(rng.choice(len(s), m, replace=False))]))
        t6 = pose6(t4)
        g = t6.copy()
        g[:2] += rng.uniform(-0.5, 0.5, 2)
        g[5] += math.radians(rng.uniform(-2.0, 2.0))
        truth.append(t6)
        guesses.append(g)
    return SearchWorkload(mp, scans, np.array(truth), np.array(guesses))


def large_map(seed=7, extent=2000.0, n_points=50_000_000, outlier_frac=0.05):
    """The large-map stress workload: the sequence generator scaled to extent x extent
    (same densities of buildings, poles and tree blobs) with a fraction of uniform outliers
    over the box [-extent/2, extent/2]^2 x [-5, 30] m, shuffled into the surface points."""
    area = (extent / 400.0) ** 2
    scene = Scene(seed, extent, int(250 * area), int(800 * area), int(300 * area))
    n_out = int(round(n_points * outlier_frac))
    pts = scene.map_points(n_points - n_out)
    rng = np.random.default_rng(seed)
    out = np.empty((n_out, 3), np.float32)
    out[:, 0] = rng.uniform(-extent / 2, extent / 2, n_out)
    out[:, 1] = rng.uniform(-extent / 2, extent / 2, n_out)
    out[:, 2] = rng.uniform(-5.0, 30.0, n_out)
    allp = np.concatenate([pts, out])
    return np.ascontiguousarray(allp[rng.permutation(len(allp))])


def crop_scan(map_points, pose, n, radius=60.0, sigma=0.02, seed=0):
    """A dense scan without ray casting: n map points within `radius` of the pose's
    position (sampled without replacement), moved into the sensor frame of `pose`
    (R = Rz(yaw)), with N(0, sigma^2) noise."""
    rng = np.random.default_rng(seed)
    d = map_points[:, :2] - np.asarray(pose[:2], np.float32)
    idx = np.nonzero((d * d).sum(1) < radius * radius)[0]
    idx = rng.choice(idx, min(n, len(idx)), replace=False)
    q = map_points[np.sort(idx)].astype(np.float64) - np.asarray(pose[:3])
    c, s = math.cos(pose[5]), math.sin(pose[5])
    local = np.stack([c * q[:, 0] + s * q[:, 1], -s * q[:, 0] + c * q[:, 1], q[:, 2]], 1)
    local += rng.normal(0, sigma, local.shape)
    return np.ascontiguousarray(local.astype(np.float32))

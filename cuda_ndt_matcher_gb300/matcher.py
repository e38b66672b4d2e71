"""NdtScanMatcher: the reference's public API (src/ndt_cuda/src/ndt.rs) over libndt_gb300.

Same names, argument meaning and error behaviour as the Rust crate:

- ``NdtScanMatcher.builder().resolution(2.0).max_iterations(30)...build()``
- ``set_target(points)``; ``align(source, initial_guess)``; ``align_gpu``;
  ``align_batch`` / ``align_batch_gpu`` (one scan, many initial poses);
  ``align_parallel_scans([(points, guess), ...])``; ``evaluate_nvtl``;
  ``evaluate_transform_probability``; ``evaluate_nvtl_batch``.

Isometries are 4x4 homogeneous matrices. As in the reference, a pose vector
[x, y, z, roll, pitch, yaw] is turned into an isometry with nalgebra's
``from_euler_angles`` (R = Rz*Ry*Rx) and back with ``euler_angles``
(src/ndt_cuda/src/optimization/types.rs:156-174), while the optimiser itself works with
R = Rx*Ry*Rz (the derivative kernels' convention). Every computation runs on the GPU
through the C ABI; ``use_gpu`` only selects which of the reference's two Newton
semantics ``align`` follows (the graph kernels when true, ``NdtOptimizer::align`` when
false).
"""
import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import capi


def pose_vector_to_isometry(pose):
    """nalgebra Isometry3::from_parts(t, UnitQuaternion::from_euler_angles(r, p, y))."""
    x, y, z, r, p, w = [float(v) for v in pose]
    sr, cr = math.sin(r), math.cos(r)
    sp, cp = math.sin(p), math.cos(p)
    sy, cy = math.sin(w), math.cos(w)
    T = np.eye(4)
    T[:3, :3] = [[cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr],
                 [sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr],
                 [-sp, cp * sr, cp * cr]]
    T[:3, 3] = [x, y, z]
    return T


def isometry_to_pose_vector(T):
    """(x, y, z) + nalgebra Rotation3::euler_angles() = (roll, pitch, yaw) for Rz*Ry*Rx."""
    T = np.asarray(T, dtype=np.float64)
    R = T[:3, :3]
    if abs(R[2, 0]) < 1.0 - np.finfo(np.float64).eps:
        roll = math.atan2(R[2, 1], R[2, 2])
        pitch = -math.asin(R[2, 0])
        yaw = math.atan2(R[1, 0], R[0, 0])
    else:  # gimbal lock, as nalgebra: yaw = 0
        yaw = 0.0
        if R[2, 0] < 0.0:
            pitch = math.pi / 2
            roll = math.atan2(R[0, 1], R[0, 2])
        else:
            pitch = -math.pi / 2
            roll = -math.atan2(R[0, 1], R[0, 2])
    return np.array([T[0, 3], T[1, 3], T[2, 3], roll, pitch, yaw], np.float64)


def translation(x, y, z):
    """Isometry3::translation(x, y, z)."""
    T = np.eye(4)
    T[:3, 3] = [x, y, z]
    return T


@dataclass
class NdtScanMatcherConfig:
    """src/ndt_cuda/src/ndt.rs:41-107 (defaults of NdtScanMatcherConfig::default)."""
    resolution: float = 2.0
    max_iterations: int = 30
    trans_epsilon: float = 0.01
    step_size: float = 0.1
    outlier_ratio: float = 0.55
    regularization: float = 0.001
    use_line_search: bool = False
    min_points_per_voxel: int = 6
    use_gpu: bool = False
    regularization_enabled: bool = False
    regularization_scale_factor: float = 0.01
    # device tuning (no counterpart in the reference)
    cluster_size: int = 0
    threads_per_cta: int = 0
    device: int = 0


@dataclass
class AlignResult:
    """src/ndt_cuda/src/ndt.rs:219-248."""
    pose: np.ndarray
    converged: bool
    score: float
    transform_probability: float
    nvtl: float
    iterations: int
    hessian: np.ndarray
    num_correspondences: int
    oscillation_count: int
    pose_vector: np.ndarray = field(default=None, repr=False)
    status: int = 0


class NdtScanMatcherBuilder:
    def __init__(self):
        self.config = NdtScanMatcherConfig()

    def _set(self, **kw):
        self.config = replace(self.config, **kw)
        return self

    def resolution(self, v):
        return self._set(resolution=float(v))

    def max_iterations(self, v):
        return self._set(max_iterations=int(v))

    def transformation_epsilon(self, v):
        return self._set(trans_epsilon=float(v))

    def step_size(self, v):
        return self._set(step_size=float(v))

    def outlier_ratio(self, v):
        return self._set(outlier_ratio=float(v))

    def regularization(self, v):
        return self._set(regularization=float(v))

    def use_line_search(self, v):
        return self._set(use_line_search=bool(v))

    def min_points_per_voxel(self, v):
        return self._set(min_points_per_voxel=int(v))

    def use_gpu(self, v):
        return self._set(use_gpu=bool(v))

    def regularization_enabled(self, v):
        return self._set(regularization_enabled=bool(v))

    def regularization_scale_factor(self, v):
        return self._set(regularization_scale_factor=float(v))

    def cluster_size(self, v):
        return self._set(cluster_size=int(v))

    def threads_per_cta(self, v):
        return self._set(threads_per_cta=int(v))

    def build(self):
        return NdtScanMatcher.with_config(self.config)


def _to_result(d, to_isometry=True):
    pose_iso = pose_vector_to_isometry(d["pose"])
    return AlignResult(pose=pose_iso, converged=d["converged"], score=d["score"],
                       transform_probability=d["transform_probability"], nvtl=d["nvtl"],
                       iterations=d["iterations"], hessian=d["hessian"],
                       num_correspondences=d["num_correspondences"],
                       oscillation_count=d["oscillation_count"], pose_vector=d["pose"],
                       status=d["status"])


class NdtScanMatcher:
    """src/ndt_cuda/src/ndt.rs:255-1321, executed by libndt_gb300 on the GPU."""

    def __init__(self, resolution=2.0):
        self._init(NdtScanMatcherConfig(resolution=float(resolution)))

    @classmethod
    def with_config(cls, config):
        self = cls.__new__(cls)
        self._init(config)
        return self

    @staticmethod
    def builder():
        return NdtScanMatcherBuilder()

    def _init(self, config):
        if config.regularization_enabled:
            raise NotImplementedError("GNSS regularisation is outside this library's scope")
        self.config = config
        self._ctx = capi.Context(
            resolution=config.resolution, max_iterations=config.max_iterations,
            trans_epsilon=config.trans_epsilon, step_size=config.step_size,
            outlier_ratio=config.outlier_ratio,
            min_points_per_voxel=config.min_points_per_voxel,
            semantics=self._semantics(config.use_gpu),
            cluster_size=config.cluster_size, threads_per_cta=config.threads_per_cta,
            device=config.device, use_line_search=int(config.use_line_search))
        self._has_target = False

    @staticmethod
    def _semantics(use_gpu):
        return capi.SEMANTICS_GPU_GRAPH if use_gpu else capi.SEMANTICS_CPU

    def _with(self, use_gpu):
        """Selects the path: the graph kernels (align_gpu) or NdtOptimizer::align. With
        use_line_search the graph path runs its parallel line search and the CPU path its
        More-Thuente search (solver.rs:268-280)."""
        want = self._semantics(use_gpu)
        if self._ctx.cfg.semantics != want:
            self._ctx.configure(semantics=want)

    def has_target(self):
        return self._has_target

    def set_target(self, points):
        pts = capi.as_xyz(points)
        self._ctx.set_target(pts)
        self._has_target = True

    def target_info(self):
        return self._ctx.map_info()

    def target_voxels(self):
        return self._ctx.map_voxels()

    def align(self, source_points, initial_guess):
        self._with(self.config.use_gpu)
        pose = isometry_to_pose_vector(initial_guess)
        return _to_result(self._ctx.align(source_points, pose))

    def align_gpu(self, source_points, initial_guess):
        self._with(True)
        pose = isometry_to_pose_vector(initial_guess)
        return _to_result(self._ctx.align(source_points, pose))

    def align_batch(self, source_points, initial_poses):
        """rayon par_iter of NdtOptimizer::align in the reference: CPU-path semantics."""
        self._with(False)
        poses = [isometry_to_pose_vector(T) for T in initial_poses]
        if not poses:
            return []
        return [_to_result(d) for d in self._ctx.align_multi_pose(source_points, poses)]

    def align_batch_gpu(self, source_points, initial_poses):
        self._with(True)
        poses = [isometry_to_pose_vector(T) for T in initial_poses]
        if not poses:
            return []
        return [_to_result(d) for d in self._ctx.align_multi_pose(source_points, poses)]

    def align_parallel_scans(self, scans):
        """align_parallel_scans: transform_probability = score / correspondences as in
        src/ndt_cuda/src/ndt.rs:1297-1316 (the NVTL is computed rather than left at 0)."""
        if not scans:
            return []
        if max(len(capi.as_xyz(p)) for p, _ in scans) == 0:
            raise capi.NdtError(-3, "All source point clouds are empty")
        self._with(True)
        pts = [p for p, _ in scans]
        poses = [isometry_to_pose_vector(T) for _, T in scans]
        out = []
        for d in self._ctx.align_batch(pts, poses):
            r = _to_result(d)
            r.transform_probability = (r.score / r.num_correspondences
                                       if r.num_correspondences > 0 else 0.0)
            out.append(r)
        return out

    def evaluate_nvtl(self, source_points, pose):
        if len(capi.as_xyz(source_points)) == 0:
            self._require_target()
            raise capi.NdtError(-3, "Source point cloud is empty")
        nvtl, _ = self._ctx.eval_batch(source_points, [np.asarray(pose)[:3, :4]])
        return float(nvtl[0])

    def evaluate_transform_probability(self, source_points, pose):
        if len(capi.as_xyz(source_points)) == 0:
            self._require_target()
            raise capi.NdtError(-3, "Source point cloud is empty")
        _, tp = self._ctx.eval_batch(source_points, [np.asarray(pose)[:3, :4]])
        return float(tp[0])

    def evaluate_nvtl_batch(self, source_points, poses):
        self._require_target()
        if len(capi.as_xyz(source_points)) == 0:
            return [0.0] * len(poses)
        if not len(poses):
            return []
        nvtl, _ = self._ctx.eval_batch(source_points, [np.asarray(T)[:3, :4] for T in poses])
        return [float(v) for v in nvtl]

    def _require_target(self):
        if not self._has_target:
            raise capi.NdtError(-2, "No target set. Call set_target() first.")

    def stats(self):
        return self._ctx.stats()

    def close(self):
        self._ctx.close()

"""ctypes binding of libndt_gb300.so (the C ABI declared in include/ndt_gb300.h).

Loading fails loudly when the library is missing; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

NDT_OK = 0
ERRORS = {
    -1: "NDT_ERR_INVALID_ARGUMENT", -2: "NDT_ERR_NO_TARGET", -3: "NDT_ERR_EMPTY_INPUT",
    -4: "NDT_ERR_NO_VOXELS", -5: "NDT_ERR_RANGE", -6: "NDT_ERR_HASH_FULL",
    -7: "NDT_ERR_PROBE_LIMIT", -8: "NDT_ERR_DEVICE", -9: "NDT_ERR_NO_DEVICE",
    -10: "NDT_ERR_CAPACITY",
}
SEMANTICS_GPU_GRAPH = 0
SEMANTICS_CPU = 1
STATUS = {0: "Converged", 1: "MaxIterations", 2: "NoCorrespondences", 3: "SingularHessian"}

# exported symbols, in the order of include/ndt_gb300.h
EXPORTS = [
    "ndt_config_default", "ndt_ctx_create", "ndt_ctx_destroy", "ndt_ctx_configure",
    "ndt_ctx_stream",
    "ndt_set_target", "ndt_set_target_device", "ndt_map_info_get", "ndt_tile_put",
    "ndt_tile_remove", "ndt_tiles_commit", "ndt_tiles_status", "ndt_map_voxels",
    "ndt_align", "ndt_align_multi_pose", "ndt_align_batch", "ndt_align_batch_device",
    "ndt_batch_submit", "ndt_batch_poll", "ndt_batch_wait",
    "ndt_autotune", "ndt_eval_batch", "ndt_batch_timings", "ndt_initial_pose_search",
    "ndt_tpe_propose",
    "ndt_pnet_config_default", "ndt_pnet_create", "ndt_pnet_destroy", "ndt_pnet_get_config",
    "ndt_pnet_add_map", "ndt_pnet_add_scan", "ndt_pnet_train", "ndt_pnet_propose",
    "ndt_pnet_debug_grad", "ndt_pnet_params", "ndt_pnet_stats_get", "ndt_learned_pose_search",
    "ndt_gemm_bf16",
    "ndt_neighbors_query", "ndt_stats_get", "ndt_stats_reset",
    "ndt_profile_enable", "ndt_debug_trace", "ndt_debug_read", "ndt_debug_queue_stall",
    "ndt_last_error_string",
    "ndt_radix_sort_pairs_u64_u32", "ndt_radix_sort_pairs_u64_u32_static",
    "ndt_detect_segments", "ndt_morton_codes",
]


class NdtError(RuntimeError):
    def __init__(self, code, msg):
        self.code = code
        super().__init__(f"{ERRORS.get(code, 'cudaError %d' % code)}: {msg}")


class Config(C.Structure):
    _fields_ = [("resolution", C.c_float), ("max_iterations", C.c_int32),
                ("trans_epsilon", C.c_double), ("step_size", C.c_double),
                ("outlier_ratio", C.c_double), ("min_points_per_voxel", C.c_int32),
                ("eigenvalue_ratio", C.c_float), ("max_neighbors", C.c_int32),
                ("semantics", C.c_int32), ("min_correspondences", C.c_int32),
                ("device", C.c_int32), ("cluster_size", C.c_int32),
                ("threads_per_cta", C.c_int32), ("hash_capacity_factor", C.c_int32),
                ("max_registers", C.c_int32), ("cell_index", C.c_int32),
                ("cuda_graph", C.c_int32), ("use_line_search", C.c_int32),
                ("work_queue", C.c_int32), ("lanes_per_point", C.c_int32),
                ("stage_points", C.c_int32)]


class Result(C.Structure):
    _fields_ = [("pose", C.c_double * 6), ("score", C.c_double),
                ("transform_probability", C.c_double), ("nvtl", C.c_double),
                ("hessian", C.c_double * 36), ("converged", C.c_int32),
                ("iterations", C.c_int32), ("num_correspondences", C.c_int32),
                ("oscillation_count", C.c_int32), ("status", C.c_int32),
                ("reserved", C.c_int32)]


class Scan(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("num_points", C.c_uint64),
                ("initial_pose", C.c_double * 6)]


class TuneResult(C.Structure):
    _fields_ = [("cluster_size", C.c_int32), ("threads_per_cta", C.c_int32),
                ("kernel_ms", C.c_double), ("aligns_per_s", C.c_double),
                ("candidates", C.c_int32), ("registers", C.c_int32),
                ("work_queue", C.c_int32), ("lanes_per_point", C.c_int32),
                ("stage_points", C.c_int32), ("reserved", C.c_int32)]


class ParticleConfig(C.Structure):
    _fields_ = [("num_particles", C.c_uint32), ("guided", C.c_uint32),
                ("xy_range", C.c_double), ("yaw_range", C.c_double),
                ("z_sigma", C.c_double), ("roll_pitch_sigma", C.c_double),
                ("seed", C.c_uint64)]


class PoseEstimate(C.Structure):
    _fields_ = [("pose", C.c_double * 6), ("initial_pose", C.c_double * 6),
                ("nvtl", C.c_double), ("score", C.c_double), ("selection_score", C.c_double),
                ("particle", C.c_int32), ("iterations", C.c_int32), ("converged", C.c_int32),
                ("reserved", C.c_int32)]


class PNetConfig(C.Structure):
    _fields_ = [("input_dim", C.c_int32), ("hidden", C.c_int32), ("hidden_layers", C.c_int32),
                ("proposals", C.c_int32), ("batch", C.c_int32), ("learning_rate", C.c_float),
                ("xy_range", C.c_float), ("yaw_weight", C.c_float), ("seed", C.c_uint64),
                ("train_batch", C.c_int32), ("reserved", C.c_int32)]


class PNetStats(C.Structure):
    _fields_ = [("inference_batches", C.c_uint64), ("queries", C.c_uint64),
                ("inference_kernel_ms", C.c_double), ("train_steps", C.c_uint64),
                ("train_ms", C.c_double)]


class MapInfo(C.Structure):
    _fields_ = [("num_points", C.c_uint64), ("num_segments", C.c_uint64),
                ("num_voxels", C.c_uint64), ("hash_capacity", C.c_uint64),
                ("max_probe", C.c_uint32), ("key_bits", C.c_uint32 * 3),
                ("min_coord", C.c_int32 * 3), ("max_coord", C.c_int32 * 3),
                ("build_ms", C.c_float), ("dense_grid_mib", C.c_float),
                ("masks_per_cell", C.c_uint32), ("reserved", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("align_launches", C.c_uint64), ("alignments", C.c_uint64),
                ("iterations", C.c_uint64), ("point_iterations", C.c_uint64),
                ("correspondences", C.c_uint64), ("align_kernel_ms", C.c_double),
                ("score_launches", C.c_uint64), ("score_kernel_ms", C.c_double),
                ("build_launches", C.c_uint64), ("build_ms", C.c_double),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("cycles_points", C.c_uint64), ("cycles_cluster_wait", C.c_uint64),
                ("cycles_control", C.c_uint64), ("cycles_broadcast", C.c_uint64),
                ("eigen_solves", C.c_uint64), ("proposal_launches", C.c_uint64),
                ("proposal_kernel_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib_path():
    return _build.CUDA_LIB


def load(build_if_missing=True):
    """Load libndt_gb300.so (built in-tree). Raises if it cannot be built or loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.CUDA_LIB
    if build_if_missing:
        _build.build_cuda()
    if not os.path.exists(path):
        raise RuntimeError(f"libndt_gb300.so not found at {path}; run __graft_entry__.build()")
    L = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "ndt_config_default": (C.c_int, [C.POINTER(Config)]),
        "ndt_ctx_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
        "ndt_ctx_destroy": (C.c_int, [P]),
        "ndt_ctx_configure": (C.c_int, [P, C.POINTER(Config)]),
        "ndt_ctx_stream": (C.c_void_p, [P]),
        "ndt_set_target": (C.c_int, [P, P, C.c_uint64]),
        "ndt_set_target_device": (C.c_int, [P, P, C.c_uint64]),
        "ndt_map_info_get": (C.c_int, [P, C.POINTER(MapInfo)]),
        "ndt_tile_put": (C.c_int, [P, C.c_uint64, P, C.c_uint64]),
        "ndt_tile_remove": (C.c_int, [P, C.c_uint64]),
        "ndt_tiles_commit": (C.c_int, [P, C.c_int32]),
        "ndt_tiles_status": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "ndt_map_voxels": (C.c_int, [P, P, P, P, P, P, C.c_uint64]),
        "ndt_align": (C.c_int, [P, P, C.c_uint64, P, C.POINTER(Result)]),
        "ndt_align_multi_pose": (C.c_int, [P, P, C.c_uint64, P, C.c_uint64, P]),
        "ndt_align_batch": (C.c_int, [P, P, C.c_uint64, P]),
        "ndt_batch_submit": (C.c_int, [P, P, C.c_uint64, C.POINTER(C.c_uint64)]),
        "ndt_batch_poll": (C.c_int, [P, C.c_uint64, C.POINTER(C.c_int32)]),
        "ndt_batch_wait": (C.c_int, [P, C.c_uint64, P]),
        "ndt_align_batch_device": (C.c_int, [P, P, P, P, C.c_uint64, P]),
        "ndt_autotune": (C.c_int, [P, P, P, P, C.c_uint64, C.c_int32, C.POINTER(TuneResult)]),
        "ndt_eval_batch": (C.c_int, [P, P, C.c_uint64, P, C.c_uint64, P, P]),
        "ndt_batch_timings": (C.c_int, [P, P, P, C.c_uint64]),
        "ndt_pnet_config_default": (C.c_int, [C.POINTER(PNetConfig)]),
        "ndt_pnet_create": (C.c_int, [C.POINTER(PNetConfig), C.c_int32, C.POINTER(C.c_void_p)]),
        "ndt_pnet_destroy": (C.c_int, [P]),
        "ndt_pnet_get_config": (C.c_int, [P, C.POINTER(PNetConfig)]),
        "ndt_pnet_add_map": (C.c_int, [P, P, C.c_uint64, C.POINTER(C.c_int32)]),
        "ndt_pnet_add_scan": (C.c_int, [P, C.c_int32, P, C.c_uint64, P, C.POINTER(C.c_int32)]),
        "ndt_pnet_train": (C.c_int, [P, C.c_uint64, P]),
        "ndt_pnet_propose": (C.c_int, [P, C.c_int32, P, C.c_uint64, P, P]),
        "ndt_pnet_debug_grad": (C.c_int, [P, P, P, C.c_uint64, P, P]),
        "ndt_pnet_params": (C.c_int, [P, P, C.POINTER(C.c_uint64), C.c_int32]),
        "ndt_pnet_stats_get": (C.c_int, [P, C.POINTER(PNetStats)]),
        "ndt_learned_pose_search": (C.c_int, [P, P, C.c_int32, P, C.c_uint64,
                                              C.POINTER(ParticleConfig), C.c_double,
                                              C.POINTER(ParticleConfig), P, P]),
        "ndt_gemm_bf16": (C.c_int, [P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]),
        "ndt_initial_pose_search": (C.c_int, [P, P, C.c_uint64, C.POINTER(ParticleConfig),
                                              P, P]),
        "ndt_tpe_propose": (C.c_int, [C.POINTER(ParticleConfig), C.c_uint64, C.c_uint64, P, P,
                                      C.c_uint64, P]),
        "ndt_neighbors_query": (C.c_int, [P, P, C.c_uint64, C.c_int32, P, P]),
        "ndt_stats_get": (C.c_int, [P, C.POINTER(Stats)]),
        "ndt_debug_queue_stall": (C.c_int, [P, C.c_uint64, C.c_int32]),
        "ndt_stats_reset": (C.c_int, [P]),
        "ndt_profile_enable": (C.c_int, [P, C.c_int]),
        "ndt_debug_trace": (C.c_int, [P, C.c_int]),
        "ndt_debug_read": (C.c_int, [P, C.c_uint64, P, C.c_int32, C.POINTER(C.c_int32)]),
        "ndt_last_error_string": (C.c_char_p, []),
        "ndt_radix_sort_pairs_u64_u32": (C.c_int, [P, P, C.c_uint64, C.c_int32, C.c_int32, P,
                                                   C.POINTER(C.c_uint64), P]),
        "ndt_radix_sort_pairs_u64_u32_static": (C.c_int, [P, P, C.c_uint64, C.c_int32,
                                                          C.c_int32, P]),
        "ndt_detect_segments": (C.c_int, [P, C.c_uint64, P, P, P, P, C.POINTER(C.c_uint64), P]),
        "ndt_morton_codes": (C.c_int, [P, C.c_uint64, C.c_float, P, P, P, P,
                                       C.POINTER(C.c_uint64), P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != NDT_OK:
        msg = _lib.ndt_last_error_string()
        raise NdtError(rc, msg.decode() if msg else "")
    return rc


def default_config(**overrides):
    cfg = Config()
    load().ndt_config_default(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def as_xyz(points):
    a = np.ascontiguousarray(np.asarray(points, dtype=np.float32).reshape(-1, 3))
    return a


def result_dict(r: Result):
    return {
        "pose": np.array(r.pose[:], dtype=np.float64),
        "score": r.score,
        "transform_probability": r.transform_probability,
        "nvtl": r.nvtl,
        "hessian": np.array(r.hessian[:], dtype=np.float64).reshape(6, 6),
        "converged": bool(r.converged),
        "iterations": r.iterations,
        "num_correspondences": r.num_correspondences,
        "oscillation_count": r.oscillation_count,
        "status": r.status,
    }



def tpe_propose(query, particle, prior, trials, num_particles=200, guided=100, xy_range=2.0,
                yaw_range=np.pi, z_sigma=0.0, roll_pitch_sigma=0.0, seed=0):
    """The TPE proposal of a guided particle (host only, no device): trials are the query's
    aligned results so far in the order they were aligned, rows (x, y, yaw, exp(-score/10))."""
    pc = ParticleConfig(num_particles=num_particles, guided=guided, xy_range=xy_range,
                        yaw_range=yaw_range, z_sigma=z_sigma, roll_pitch_sigma=roll_pitch_sigma,
                        seed=seed)
    t = np.ascontiguousarray(np.asarray(trials, np.float64).reshape(-1, 4))
    pr = np.ascontiguousarray(prior, np.float64)
    out = np.zeros(6)
    check(load().ndt_tpe_propose(C.byref(pc), query, particle, pr.ctypes.data, t.ctypes.data,
                                 len(t), out.ctypes.data))
    return out

class Context:
    """Thin owner of an ndt_ctx*: every method is one C-ABI call."""

    def __init__(self, **cfg):
        self.lib = load()
        self.cfg = default_config(**cfg)
        h = C.c_void_p()
        check(self.lib.ndt_ctx_create(C.byref(self.cfg), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.ndt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def configure(self, **overrides):
        for k, v in overrides.items():
            setattr(self.cfg, k, v)
        check(self.lib.ndt_ctx_configure(self.h, C.byref(self.cfg)))

    @property
    def stream(self):
        return self.lib.ndt_ctx_stream(self.h)

    def set_target(self, points):
        p = as_xyz(points)
        check(self.lib.ndt_set_target(self.h, p.ctypes.data, len(p)))

    def tile_put(self, tile_id, points):
        p = as_xyz(points)
        check(self.lib.ndt_tile_put(self.h, tile_id, p.ctypes.data, len(p)))

    def tile_remove(self, tile_id):
        check(self.lib.ndt_tile_remove(self.h, tile_id))

    def tiles_commit(self, wait=True):
        check(self.lib.ndt_tiles_commit(self.h, 1 if wait else 0))

    def tiles_status(self):
        nt, npnt = C.c_uint64(), C.c_uint64()
        pend, rc, ms, put = C.c_int32(), C.c_int32(), C.c_float(), C.c_float()
        check(self.lib.ndt_tiles_status(self.h, C.byref(nt), C.byref(npnt), C.byref(pend),
                                        C.byref(rc), C.byref(ms), C.byref(put)))
        return {"tiles": nt.value, "points": npnt.value, "pending": bool(pend.value),
                "last_rc": rc.value, "build_ms": ms.value, "put_ms": put.value}

    def set_target_device(self, ptr, n):
        check(self.lib.ndt_set_target_device(self.h, ptr, n))

    def map_info(self):
        mi = MapInfo()
        check(self.lib.ndt_map_info_get(self.h, C.byref(mi)))
        return mi

    def map_voxels(self):
        v = int(self.map_info().num_voxels)
        coords = np.zeros((v, 3), np.int32)
        means = np.zeros((v, 3), np.float32)
        covs = np.zeros((v, 9), np.float32)
        icovs = np.zeros((v, 9), np.float32)
        counts = np.zeros(v, np.uint32)
        check(self.lib.ndt_map_voxels(self.h, coords.ctypes.data, means.ctypes.data,
                                      covs.ctypes.data, icovs.ctypes.data, counts.ctypes.data,
                                      v))
        return coords, means, covs, icovs, counts

    def align(self, points, pose):
        p = as_xyz(points)
        pose = np.ascontiguousarray(pose, np.float64)
        r = Result()
        check(self.lib.ndt_align(self.h, p.ctypes.data, len(p), pose.ctypes.data, C.byref(r)))
        return result_dict(r)

    def align_multi_pose(self, points, poses):
        p = as_xyz(points)
        poses = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 6))
        res = (Result * len(poses))()
        check(self.lib.ndt_align_multi_pose(self.h, p.ctypes.data, len(p), poses.ctypes.data,
                                            len(poses), res))
        return [result_dict(r) for r in res]

    @staticmethod
    def _scan_array(scans, poses):
        scans = [as_xyz(s) for s in scans]
        m = len(scans)
        arr = (Scan * m)()
        for i, (s, pose) in enumerate(zip(scans, poses)):
            arr[i].xyz = s.ctypes.data
            arr[i].num_points = len(s)
            for k in range(6):
                arr[i].initial_pose[k] = float(pose[k])
        return arr, m, scans

    def align_batch(self, scans, poses):
        arr, m, keep = self._scan_array(scans, poses)
        res = (Result * m)()
        check(self.lib.ndt_align_batch(self.h, arr, m, res))
        return [result_dict(r) for r in res]

    def batch_submit(self, scans, poses):
        """Queues a batch (AsyncBatchPipeline::submit); returns (ticket, number of scans)."""
        arr, m, keep = self._scan_array(scans, poses)
        t = C.c_uint64()
        check(self.lib.ndt_batch_submit(self.h, arr, m, C.byref(t)))
        return t.value, m

    def batch_poll(self, ticket):
        ready = C.c_int32()
        check(self.lib.ndt_batch_poll(self.h, ticket[0], C.byref(ready)))
        return bool(ready.value)

    def batch_wait(self, ticket):
        res = (Result * max(ticket[1], 1))()
        check(self.lib.ndt_batch_wait(self.h, ticket[0], res))
        return [result_dict(r) for r in res[:ticket[1]]]

    def align_batch_raw(self, scan_array, results):
        """Hot-path form: prebuilt (Scan * m) and (Result * m) arrays, no conversion."""
        check(self.lib.ndt_align_batch(self.h, scan_array, len(scan_array), results))

    def align_batch_device(self, d_xyz, offsets, poses):
        offsets = np.ascontiguousarray(offsets, np.uint64)
        poses = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 6))
        m = len(poses)
        res = (Result * m)()
        check(self.lib.ndt_align_batch_device(self.h, d_xyz, offsets.ctypes.data,
                                              poses.ctypes.data, m, res))
        return [result_dict(r) for r in res]

    def autotune(self, d_xyz, offsets, poses, repeats=2):
        """Times the launch-shape candidates on a device-resident batch; returns the winner."""
        offsets = np.ascontiguousarray(offsets, np.uint64)
        poses = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 6))
        r = TuneResult()
        check(self.lib.ndt_autotune(self.h, d_xyz, offsets.ctypes.data, poses.ctypes.data,
                                    len(poses), repeats, C.byref(r)))
        return {"cluster_size": r.cluster_size, "threads_per_cta": r.threads_per_cta,
                "kernel_ms": r.kernel_ms, "aligns_per_s": r.aligns_per_s,
                "candidates": r.candidates, "registers": r.registers,
                "work_queue": r.work_queue, "lanes_per_point": r.lanes_per_point,
                "stage_points": r.stage_points}

    def batch_timings(self, n):
        """Start / finish (ms, device clock) of each alignment of the last call."""
        start = np.zeros(n)
        finish = np.zeros(n)
        check(self.lib.ndt_batch_timings(self.h, start.ctypes.data, finish.ctypes.data, n))
        return start, finish

    def initial_pose_search(self, queries, priors, num_particles=200, xy_range=2.0,
                            yaw_range=np.pi, z_sigma=0.0, roll_pitch_sigma=0.0, seed=0,
                            return_particles=False, guided=0):
        """Batched multi-particle search; returns one estimate dict per query (and, when
        asked, every particle's result, query-major). guided: the last particles of each
        query that are TPE-guided (the reference's guided phase)."""
        qs = [as_xyz(q) for q in queries]
        m = len(qs)
        arr = (Scan * m)()
        for i, (s, pose) in enumerate(zip(qs, priors)):
            arr[i].xyz = s.ctypes.data
            arr[i].num_points = len(s)
            for k in range(6):
                arr[i].initial_pose[k] = float(pose[k])
        pc = ParticleConfig(num_particles=num_particles, guided=guided, xy_range=xy_range,
                            yaw_range=yaw_range, z_sigma=z_sigma,
                            roll_pitch_sigma=roll_pitch_sigma, seed=seed)
        est = (PoseEstimate * m)()
        parts = (Result * (m * num_particles))() if return_particles else None
        check(self.lib.ndt_initial_pose_search(self.h, arr, m, C.byref(pc), est, parts))
        out = [{"pose": np.array(e.pose), "initial_pose": np.array(e.initial_pose),
                "nvtl": e.nvtl, "score": e.score, "selection_score": e.selection_score,
                "particle": e.particle, "iterations": e.iterations,
                "converged": bool(e.converged)} for e in est]
        if return_particles:
            return out, [result_dict(r) for r in parts]
        return out

    def eval_batch(self, points, T34):
        p = as_xyz(points)
        T = np.ascontiguousarray(np.asarray(T34, np.float64).reshape(-1, 12))
        m = len(T)
        nvtl = np.zeros(m)
        tp = np.zeros(m)
        check(self.lib.ndt_eval_batch(self.h, p.ctypes.data, len(p), T.ctypes.data, m,
                                      nvtl.ctypes.data, tp.ctypes.data))
        return nvtl, tp

    def neighbors(self, q, max_nb=8):
        q = as_xyz(q)
        idx = np.zeros((len(q), max_nb), np.int32)
        cnt = np.zeros(len(q), np.int32)
        check(self.lib.ndt_neighbors_query(self.h, q.ctypes.data, len(q), max_nb,
                                           idx.ctypes.data, cnt.ctypes.data))
        return idx, cnt

    def debug_queue_stall(self, limit_ns, withhold_next=False):
        """Test hook: the work-queue kernel's no-progress limit, and (withhold_next) a next
        launch whose chunks all start out claimed, so the limit runs out."""
        check(self.lib.ndt_debug_queue_stall(self.h, int(limit_ns), 1 if withhold_next else 0))

    def trace(self, enable=True):
        check(self.lib.ndt_debug_trace(self.h, 1 if enable else 0))

    def read_trace(self, index):
        out = np.zeros((self.cfg.max_iterations, 48))
        n = C.c_int32()
        check(self.lib.ndt_debug_read(self.h, index, out.ctypes.data, len(out), C.byref(n)))
        return out[:n.value]

    def stats(self):
        s = Stats()
        check(self.lib.ndt_stats_get(self.h, C.byref(s)))
        return s.as_dict()

    def stats_reset(self):
        check(self.lib.ndt_stats_reset(self.h))

    def learned_pose_search(self, net, map_id, queries, coarse, nvtl_threshold=2.3,
                            fallback=None, refine=None):
        """Proposal network + NDT refinement; `refine` (a dict of particle settings: particles
        around each query's best proposal result, aligned as a second round); plain particle
        search below the NVTL threshold when `fallback` is a dict of initial_pose_search
        particle settings."""
        def pcfg(d):
            f = dict(num_particles=200, xy_range=2.0, yaw_range=np.pi, z_sigma=0.0,
                     roll_pitch_sigma=0.0, seed=0)
            f.update(d)
            return ParticleConfig(**f)
        qs = [as_xyz(q) for q in queries]
        m = len(qs)
        arr = (Scan * m)()
        for i, (s, pose) in enumerate(zip(qs, coarse)):
            arr[i].xyz = s.ctypes.data
            arr[i].num_points = len(s)
            for k in range(6):
                arr[i].initial_pose[k] = float(pose[k])
        pc = pcfg(fallback) if fallback is not None else None
        rf = pcfg(refine) if refine is not None else None
        est = (PoseEstimate * m)()
        used = np.zeros(m, np.int32)
        check(self.lib.ndt_learned_pose_search(self.h, net.h, map_id, arr, m,
                                               C.byref(rf) if rf is not None else None,
                                               nvtl_threshold,
                                               C.byref(pc) if pc is not None else None, est,
                                               used.ctypes.data))
        return [{"pose": np.array(e.pose), "initial_pose": np.array(e.initial_pose),
                 "nvtl": e.nvtl, "score": e.score, "selection_score": e.selection_score,
                 "particle": e.particle, "iterations": e.iterations,
                 "converged": bool(e.converged), "fallback": bool(u)}
                for e, u in zip(est, used)]


class PNet:
    """The learned initial-pose proposal network (libndt_gb300 ndt_pnet_*)."""

    def __init__(self, device=0, **cfg):
        self.lib = load()
        self.cfg = PNetConfig()
        check(self.lib.ndt_pnet_config_default(C.byref(self.cfg)))
        for k, v in cfg.items():
            setattr(self.cfg, k, v)
        h = C.c_void_p()
        check(self.lib.ndt_pnet_create(C.byref(self.cfg), device, C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.ndt_pnet_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_map(self, points):
        p = as_xyz(points)
        mid = C.c_int32()
        check(self.lib.ndt_pnet_add_map(self.h, p.ctypes.data, len(p), C.byref(mid)))
        return mid.value

    def add_scan(self, map_id, points, pose):
        p = as_xyz(points)
        pose = np.ascontiguousarray(pose, np.float64)
        sid = C.c_int32()
        check(self.lib.ndt_pnet_add_scan(self.h, map_id, p.ctypes.data, len(p),
                                         pose.ctypes.data, C.byref(sid)))
        return sid.value

    def train(self, steps, record_loss=True):
        """steps Adam steps; with record_loss the per-step mean loss is returned (read back
        after every step), else None."""
        if not record_loss:
            check(self.lib.ndt_pnet_train(self.h, steps, None))
            return None
        loss = np.zeros(steps, np.float32)
        check(self.lib.ndt_pnet_train(self.h, steps, loss.ctypes.data))
        return loss

    def stats(self):
        st = PNetStats()
        check(self.lib.ndt_pnet_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def propose(self, map_id, queries, coarse):
        qs = [as_xyz(q) for q in queries]
        m = len(qs)
        arr = (Scan * m)()
        for i, (s, pose) in enumerate(zip(qs, coarse)):
            arr[i].xyz = s.ctypes.data
            arr[i].num_points = len(s)
            for k in range(6):
                arr[i].initial_pose[k] = float(pose[k])
        P = self.cfg.proposals
        poses = np.zeros((m, P, 6))
        logits = np.zeros((m, P))
        check(self.lib.ndt_pnet_propose(self.h, map_id, arr, m, poses.ctypes.data,
                                        logits.ctypes.data))
        return poses, logits

    def params(self):
        n = C.c_uint64()
        check(self.lib.ndt_pnet_params(self.h, None, C.byref(n), 0))
        out = np.zeros(n.value, np.float32)
        check(self.lib.ndt_pnet_params(self.h, out.ctypes.data, C.byref(n), 0))
        return out

    def set_params(self, values):
        v = np.ascontiguousarray(values, np.float32)
        n = C.c_uint64(len(v))
        check(self.lib.ndt_pnet_params(self.h, v.ctypes.data, C.byref(n), 1))

    def debug_grad(self, x, targets):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        n = C.c_uint64()
        check(self.lib.ndt_pnet_params(self.h, None, C.byref(n), 0))
        g = np.zeros(n.value, np.float32)
        loss = C.c_float()
        check(self.lib.ndt_pnet_debug_grad(self.h, x.ctypes.data, t.ctypes.data, len(x),
                                           C.byref(loss), g.ctypes.data))
        return loss.value, g


def gemm_bf16(a, b, splits=1):
    """D = A B^T for torch bf16 CUDA tensors A [m x k], B [n x k] (k % 64 == 0); with
    splits > 1 the split-K partial products are computed and summed here."""
    import torch
    m, k = a.shape
    n = b.shape[0]
    d = torch.empty((splits, m, n), dtype=torch.float32, device=a.device)
    check(load().ndt_gemm_bf16(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                               C.c_void_p(d.data_ptr()), m, n, k, splits, None))
    return d.sum(0) if splits > 1 else d[0]

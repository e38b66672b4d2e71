"""The reference's own graph-path CUDA kernels, run on the GPU as a checker (test
infrastructure: only tests load it).

`oracle/_ref/*.cubin` are the reference's `ndt_graph_kernels.cu` and `voxel_hash.cu`
compiled unmodified (oracle/build.py); `oracle/ref_graph.c` is the host side, a restatement
of `FullGpuPipelineV2::optimize` (src/ndt_cuda/src/optimization/full_gpu_pipeline_v2.rs:487-669)
over the CUDA driver API. The result is what the reference's GPU `align` returns for the same
voxel map, scan and initial pose (FP32 state, FP32 atomic reductions: it varies slightly run
to run, and its spread is measured beside every comparison).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))


def available():
    """True when the cubins exist (they are built where the reference sources are, and
    travel with the repository copy)."""
    return all(os.path.exists(os.path.join(_build.REF_DIR, c)) for c in _build.REF_CUBINS)


class RefGraph:
    """One map at a time; align() runs K1..K5 until converged or max_iterations."""

    def __init__(self):
        lib = C.CDLL(_build.build_ref_driver())
        lib.rg_error.restype = C.c_char_p
        lib.rg_open.argtypes = [C.c_char_p]
        lib.rg_set_map.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_float]
        lib.rg_align.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_float, C.c_float,
                                 C.c_double, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                 C.c_float, C.c_void_p, C.c_void_p]
        lib.rg_query.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        lib.rg_eval.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_float, C.c_float,
                                C.c_void_p]
        self.lib = lib
        self._check(lib.rg_open(_build.REF_DIR.encode()))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("reference kernels: " + self.lib.rg_error().decode())

    def set_map(self, means, icovs, resolution=2.0):
        means = np.ascontiguousarray(means, np.float32).reshape(-1, 3)
        icovs = np.ascontiguousarray(icovs, np.float32).reshape(-1, 9)
        assert len(means) == len(icovs)
        self._check(self.lib.rg_set_map(means.ctypes.data, icovs.ctypes.data, len(means),
                                         float(resolution)))

    def align(self, points, pose, d1, d2, trans_epsilon=0.01, max_iterations=30,
              line_search=False, step_size=0.1, ls_mu=1e-4, ls_nu=0.9, debug=False):
        """With debug, the result also holds K5's per-iteration records ("debug": iteration,
        score, pose before, gradient, Hessian upper triangle, step, alpha, correspondences,
        direction reversed, pose after; 50 values per iteration)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        pose = np.ascontiguousarray(pose, np.float64)
        out = np.zeros(48, np.float32)
        dbg = np.zeros((max(int(max_iterations), 1), 50), np.float32) if debug else None
        self._check(self.lib.rg_align(pts.ctypes.data, len(pts), pose.ctypes.data,
                                      float(d1), float(d2), float(trans_epsilon),
                                      int(max_iterations), int(bool(line_search)),
                                      float(step_size), float(ls_mu), float(ls_nu),
                                      out.ctypes.data,
                                      dbg.ctypes.data if debug else None))
        o = out.astype(np.float64)
        # OutputOffset (src/cuda_ffi/csrc/ndt_graph_common.cuh:90-101), parsed as
        # full_gpu_pipeline_v2.rs:626-646 does
        return {"pose": o[:6].copy(), "iterations": int(out[6]), "converged": bool(out[7] > 0.5),
                "score": o[8], "hessian": o[9:45].reshape(6, 6),
                "num_correspondences": int(out[45]), "oscillation_count": int(out[46]),
                "avg_alpha": o[47],
                "debug": dbg[:int(out[6])].astype(np.float64) if debug else None}

    def evaluate(self, points, pose, d1, d2):
        """The reference's K2 at one pose: score, gradient (6), Hessian (6x6, from its
        upper triangle) and correspondences."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        pose = np.ascontiguousarray(pose, np.float64)
        red = np.zeros(29, np.float32)
        self._check(self.lib.rg_eval(pts.ctypes.data, len(pts), pose.ctypes.data, float(d1),
                                     float(d2), red.ctypes.data))
        r = red.astype(np.float64)
        H = np.zeros((6, 6))
        H[np.triu_indices(6)] = r[7:28]
        H = H + np.triu(H, 1).T
        return r[0], r[1:7].copy(), H, int(red[28])

    def query(self, q):
        """The reference's 27-cell hash query (radius = resolution, at most 8): voxel indices
        (n x 8, -1 padded) and counts."""
        q = np.ascontiguousarray(q, np.float32).reshape(-1, 3)
        idx = np.zeros((len(q), 8), np.int32)
        cnt = np.zeros(len(q), np.uint32)
        self._check(self.lib.rg_query(q.ctypes.data, len(q), idx.ctypes.data, cnt.ctypes.data))
        return idx, cnt.astype(np.int32)

    def close(self):
        self.lib.rg_close()

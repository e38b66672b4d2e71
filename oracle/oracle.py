"""ctypes wrapper over the oracle library (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs as the oracle
and as the timed CPU baseline. The GPU product never imports this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class OrResult(C.Structure):
    _fields_ = [("pose", C.c_double * 6), ("score", C.c_double),
                ("transform_probability", C.c_double), ("nvtl", C.c_double),
                ("hessian", C.c_double * 36), ("converged", C.c_int32),
                ("iterations", C.c_int32), ("num_correspondences", C.c_int32),
                ("oscillation_count", C.c_int32), ("status", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self):
        return {
            "pose": np.array(self.pose[:], dtype=np.float64),
            "score": self.score,
            "transform_probability": self.transform_probability,
            "nvtl": self.nvtl,
            "hessian": np.array(self.hessian[:], dtype=np.float64).reshape(6, 6),
            "converged": bool(self.converged),
            "iterations": self.iterations,
            "num_correspondences": self.num_correspondences,
            "oscillation_count": self.oscillation_count,
            "status": self.status,
        }


class OrConfig(C.Structure):
    _fields_ = [("resolution", C.c_double), ("max_iterations", C.c_int32),
                ("max_neighbors", C.c_int32), ("trans_epsilon", C.c_double),
                ("step_size", C.c_double), ("outlier_ratio", C.c_double),
                ("min_correspondences", C.c_int32), ("ls_candidates", C.c_int32),
                ("ls_mu", C.c_double), ("ls_nu", C.c_double)]


def config(resolution=2.0, max_iterations=30, max_neighbors=8, trans_epsilon=0.01,
           step_size=0.1, outlier_ratio=0.55, min_correspondences=10, ls_candidates=0,
           ls_mu=1e-4, ls_nu=0.9):
    """ls_candidates > 0 turns on the graph path's parallel line search (the reference
    pipeline uses 8 candidates, Armijo 1e-4, curvature 0.9: full_gpu_pipeline_v2.rs:101-113,
    566-567)."""
    return OrConfig(resolution, max_iterations, max_neighbors, trans_epsilon, step_size,
                    outlier_ratio, min_correspondences, ls_candidates, ls_mu, ls_nu)


MT_FN = C.CFUNCTYPE(C.c_int, C.c_double, C.c_void_p, C.POINTER(C.c_double),
                    C.POINTER(C.c_double))


def mt_search(score_and_derivative, score0, deriv0, initial, step_min=1e-9, step_max=0.1,
              mu=1e-4, nu=0.9, max_iterations=10):
    """The CPU path's More-Thuente line search (more_thuente_search) on a Python function
    alpha -> (score, directional derivative); returns (step, converged, evaluations)."""
    def cb(alpha, _ctx, sc, dr):
        s, d = score_and_derivative(alpha)
        sc[0] = s
        dr[0] = d
        return 0
    fn = MT_FN(cb)
    conv, ev = C.c_int32(), C.c_int32()
    a = lib().or_mt_search(fn, None, score0, deriv0, initial, step_min, step_max, mu, nu,
                           max_iterations, C.byref(conv), C.byref(ev))
    return a, bool(conv.value), ev.value


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
        sig = {
            "or_gauss_params": (None, [C.c_double, C.c_double, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
            "or_voxel_coord": (None, [f32p, C.c_float, i32p]),
            "or_morton_encode": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_uint32]),
            "or_morton_decode": (None, [C.c_uint64, C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
            "or_morton_codes_ref": (None, [f32p, C.c_size_t, C.c_float, u64p, f32p]),
            "or_morton_codes_coord": (C.c_int, [f32p, C.c_size_t, C.c_float, u64p, i32p]),
            "or_radix_sort_pairs": (None, [u64p, u32p, C.c_size_t]),
            "or_detect_segments": (C.c_size_t, [u64p, C.c_size_t, u32p, u32p]),
            "or_grid_build": (P, [f32p, C.c_size_t, C.c_float, C.c_int, C.c_float, C.c_int]),
            "or_grid_free": (None, [P]),
            "or_grid_size": (C.c_size_t, [P]),
            "or_grid_copy": (None, [P, i32p, f32p, f32p, f32p, u32p, f32p]),
            "or_grid_hash_capacity": (C.c_uint32, [P]),
            "or_pack_key": (C.c_int64, [C.c_int32, C.c_int32, C.c_int32]),
            "or_hash_slot": (C.c_uint32, [C.c_int64, C.c_uint32]),
            "or_grid_lookup": (C.c_int32, [P, C.c_int32, C.c_int32, C.c_int32]),
            "or_query_gpu_sem": (None, [P, f32p, C.c_size_t, C.c_int, i32p, i32p]),
            "or_radius_search": (C.c_int, [P, f32p, C.c_float, i32p, C.c_int]),
            "or_derivatives_cpu": (None, [P, f32p, C.c_size_t, f64p, C.c_double, C.c_double,
                                          C.POINTER(C.c_double), f64p, f64p,
                                          C.POINTER(C.c_int32)]),
            "or_derivatives_gpu_sem": (None, [P, f32p, C.c_size_t, f64p, C.c_double,
                                              C.c_double, C.c_int, C.POINTER(C.c_double),
                                              f64p, f64p, C.POINTER(C.c_int32)]),
            "or_newton_step_nd": (C.c_int, [f64p, f64p, C.c_double, C.c_double, f64p]),
            "or_jacobi_svd_solve": (C.c_int, [f64p, f64p, f64p]),
            "or_align_cpu": (None, [P, f32p, C.c_size_t, f64p, C.POINTER(OrConfig),
                                    C.POINTER(OrResult)]),
            "or_align_gpu_sem": (None, [P, f32p, C.c_size_t, f64p, C.POINTER(OrConfig),
                                        C.POINTER(OrResult)]),
            "or_align_gpu_sem_trace": (None, [P, f32p, C.c_size_t, f64p, C.POINTER(OrConfig),
                                              C.POINTER(OrResult), f64p]),
            "or_align_cpu_trace": (None, [P, f32p, C.c_size_t, f64p, C.POINTER(OrConfig),
                                          C.POINTER(OrResult), f64p]),
            "or_align_batch": (None, [P, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), f64p,
                                      C.c_size_t, C.POINTER(OrConfig), C.c_int, C.c_int,
                                      C.POINTER(OrResult)]),
            "or_nvtl": (C.c_double, [P, f32p, C.c_size_t, f64p, C.c_double, C.c_double,
                                     C.c_double]),
            "or_score_gpu_sem": (None, [P, f32p, C.c_size_t, f64p, C.c_double, C.c_double,
                                        C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_int32)]),
            "or_pose_to_T34_xyz": (None, [f64p, f64p]),
            "or_pose_to_T34_zyx": (None, [f64p, f64p]),
            "or_eigen_sym3": (None, [f64p, f64p, f64p]),
            "or_eigen_sym6": (None, [f64p, f64p, f64p]),
            "or_mt_search": (C.c_double, [MT_FN, P, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_int32, C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))


def gauss_params(resolution=2.0, outlier_ratio=0.55):
    d1, d2 = C.c_double(), C.c_double()
    lib().or_gauss_params(resolution, outlier_ratio, C.byref(d1), C.byref(d2))
    return d1.value, d2.value


def voxel_coord(p, res):
    out = np.zeros(3, np.int32)
    lib().or_voxel_coord(np.ascontiguousarray(p, np.float32), res, out)
    return out


def morton_encode(x, y, z):
    return int(lib().or_morton_encode(x, y, z))


def morton_decode(code):
    x, y, z = C.c_uint32(), C.c_uint32(), C.c_uint32()
    lib().or_morton_decode(code, C.byref(x), C.byref(y), C.byref(z))
    return x.value, y.value, z.value


def morton_codes_ref(pts, res):
    pts = _f32(pts)
    codes = np.zeros(len(pts), np.uint64)
    gmin = np.zeros(3, np.float32)
    lib().or_morton_codes_ref(pts, len(pts), res, codes, gmin)
    return codes, gmin


def morton_codes_coord(pts, res):
    pts = _f32(pts)
    codes = np.zeros(len(pts), np.uint64)
    mn = np.zeros(3, np.int32)
    ok = lib().or_morton_codes_coord(pts, len(pts), res, codes, mn)
    return codes, mn, bool(ok)


def radix_sort_pairs(keys, vals):
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib().or_radix_sort_pairs(k, v, len(k))
    return k, v


def detect_segments(sorted_codes):
    s = np.ascontiguousarray(sorted_codes, np.uint64)
    ids = np.zeros(max(len(s), 1), np.uint32)
    starts = np.zeros(max(len(s), 1), np.uint32)
    n = lib().or_detect_segments(s, len(s), ids, starts)
    return ids[:len(s)], starts[:n], int(n)


class Grid:
    """Oracle voxel grid (Morton-ordered valid voxels + reference-semantics hash)."""

    def __init__(self, pts, res=2.0, min_points=6, ratio=0.01, centered=True):
        self.pts = _f32(pts)
        self.res = float(res)
        self.h = lib().or_grid_build(self.pts, len(self.pts), res, min_points, ratio,
                                     1 if centered else 0)
        if not self.h:
            raise ValueError("voxel coordinate range exceeds 21 bits per axis")
        n = lib().or_grid_size(self.h)
        self.n = int(n)
        self.coords = np.zeros((max(n, 1), 3), np.int32)
        self.means = np.zeros((max(n, 1), 3), np.float32)
        self.covs = np.zeros((max(n, 1), 9), np.float32)
        self.icovs = np.zeros((max(n, 1), 9), np.float32)
        self.counts = np.zeros(max(n, 1), np.uint32)
        self.paxes = np.zeros((max(n, 1), 3), np.float32)
        lib().or_grid_copy(self.h, self.coords, self.means, self.covs, self.icovs,
                           self.counts, self.paxes)
        for a in ("coords", "means", "covs", "icovs", "counts", "paxes"):
            setattr(self, a, getattr(self, a)[:n])
        self.capacity = int(lib().or_grid_hash_capacity(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_grid_free(self.h)
            self.h = None

    def lookup(self, gx, gy, gz):
        return int(lib().or_grid_lookup(self.h, gx, gy, gz))

    def query_gpu_sem(self, q, max_nb=8):
        q = _f32(q)
        idx = np.zeros((len(q), max_nb), np.int32)
        cnt = np.zeros(len(q), np.int32)
        lib().or_query_gpu_sem(self.h, q, len(q), max_nb, idx, cnt)
        return idx, cnt

    def radius_search(self, q, radius):
        out = np.zeros(64, np.int32)
        k = lib().or_radius_search(self.h, np.ascontiguousarray(q, np.float32), radius, out, 64)
        return out[:min(k, 64)]

    def derivatives(self, src, pose, semantics="gpu", max_nb=8, resolution=None,
                    outlier_ratio=0.55):
        d1, d2 = gauss_params(resolution or self.res, outlier_ratio)
        src = _f32(src)
        pose = np.ascontiguousarray(pose, np.float64)
        sc = C.c_double()
        nc = C.c_int32()
        g = np.zeros(6)
        H = np.zeros(36)
        if semantics == "gpu":
            lib().or_derivatives_gpu_sem(self.h, src, len(src), pose, d1, d2, max_nb,
                                         C.byref(sc), g, H, C.byref(nc))
        else:
            lib().or_derivatives_cpu(self.h, src, len(src), pose, d1, d2, C.byref(sc), g, H,
                                     C.byref(nc))
        return sc.value, g, H.reshape(6, 6), nc.value

    def align(self, src, pose, semantics="gpu", **cfg):
        c = config(resolution=self.res, **cfg)
        r = OrResult()
        src = _f32(src)
        pose = np.ascontiguousarray(pose, np.float64)
        fn = lib().or_align_gpu_sem if semantics == "gpu" else lib().or_align_cpu
        fn(self.h, src, len(src), pose, C.byref(c), C.byref(r))
        return r.as_dict()

    def align_trace(self, src, pose, semantics="gpu", **cfg):
        """Alignment with the per-iteration trace (48 doubles per iteration: it, score,
        correspondences, pose before the step, gradient, Hessian upper triangle, ...)."""
        c = config(resolution=self.res, **cfg)
        r = OrResult()
        src = _f32(src)
        tr = np.full((c.max_iterations, 48), np.nan)
        fn = lib().or_align_gpu_sem_trace if semantics == "gpu" else lib().or_align_cpu_trace
        fn(self.h, src, len(src), np.ascontiguousarray(pose, np.float64), C.byref(c),
           C.byref(r), tr)
        return r.as_dict(), tr[~np.isnan(tr[:, 0])]

    def align_batch(self, scans, poses, semantics="gpu", nthreads=0, **cfg):
        c = config(resolution=self.res, **cfg)
        scans = [_f32(s) for s in scans]
        m = len(scans)
        ptrs = (C.c_void_p * m)(*[s.ctypes.data for s in scans])
        ns = (C.c_size_t * m)(*[len(s) for s in scans])
        poses = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(m, 6))
        res = (OrResult * m)()
        lib().or_align_batch(self.h, ptrs, ns, poses, m, C.byref(c),
                             0 if semantics == "gpu" else 1, nthreads, res)
        return [r.as_dict() for r in res]

    def nvtl(self, src, T34, outlier_ratio=0.55):
        d1, d2 = gauss_params(self.res, outlier_ratio)
        src = _f32(src)
        return lib().or_nvtl(self.h, src, len(src), np.ascontiguousarray(T34, np.float64).ravel(),
                             self.res, d1, d2)

    def score_gpu_sem(self, src, T34, max_nb=8, outlier_ratio=0.55):
        d1, d2 = gauss_params(self.res, outlier_ratio)
        src = _f32(src)
        sc = C.c_double()
        nc = C.c_int32()
        lib().or_score_gpu_sem(self.h, src, len(src),
                               np.ascontiguousarray(T34, np.float64).ravel(), d1, d2, max_nb,
                               C.byref(sc), C.byref(nc))
        return sc.value, nc.value


def pose_T34_xyz(pose):
    T = np.zeros(12)
    lib().or_pose_to_T34_xyz(np.ascontiguousarray(pose, np.float64), T)
    return T.reshape(3, 4)


def pose_T34_zyx(pose):
    T = np.zeros(12)
    lib().or_pose_to_T34_zyx(np.ascontiguousarray(pose, np.float64), T)
    return T.reshape(3, 4)


def newton_step_nd(g, H, min_eig=-1e-3, tol=1e-10):
    x = np.zeros(6)
    ok = lib().or_newton_step_nd(np.ascontiguousarray(g, np.float64),
                                 np.ascontiguousarray(H, np.float64).ravel(), min_eig, tol, x)
    return x if ok else None


def jacobi_svd_solve(H, g):
    x = np.zeros(6)
    ok = lib().or_jacobi_svd_solve(np.ascontiguousarray(H, np.float64).ravel(),
                                   np.ascontiguousarray(g, np.float64), x)
    return x, bool(ok)


def eigen_sym(a):
    a = np.ascontiguousarray(a, np.float64)
    n = a.shape[0]
    ev = np.zeros(n)
    V = np.zeros(n * n)
    (lib().or_eigen_sym3 if n == 3 else lib().or_eigen_sym6)(a.ravel(), ev, V)
    return ev, V.reshape(n, n)


# ---------------------------------------------------------------------------------------
# Initial-pose search (estimate_initial_pose + select_best_particle,
# src/cuda_ndt_matcher/src/initial_pose.rs:115-460, src/cuda_ndt_matcher/src/particle.rs:36-42)
# ---------------------------------------------------------------------------------------
_M64 = (1 << 64) - 1


def _splitmix64(state):
    state = (state + 0x9E3779B97F4A7C15) & _M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return state, z ^ (z >> 31)


def particle(prior, q, k, xy_range=2.0, yaw_range=np.pi, z_sigma=0.0, roll_pitch_sigma=0.0,
             seed=0):
    """Starting pose of particle k of query q: SplitMix64 stream seeded by (seed, q, k);
    x, y + U(-xy_range, xy_range), yaw + U(-yaw_range, yaw_range), then z, roll, pitch +
    N(0, sigma^2) by Box-Muller."""
    s = (seed ^ ((0x9E3779B97F4A7C15 * (q + 1)) & _M64) ^ ((0xD1B54A32D192ED03 * (k + 1)) & _M64))
    s, _ = _splitmix64(s)

    def unit():
        nonlocal s
        s, z = _splitmix64(s)
        return (z >> 11) * 2.0 ** -53

    p = np.array(prior, dtype=np.float64).copy()
    p[0] += (2.0 * unit() - 1.0) * xy_range
    p[1] += (2.0 * unit() - 1.0) * xy_range
    p[5] += (2.0 * unit() - 1.0) * yaw_range
    for sig, d in ((z_sigma, 2), (roll_pitch_sigma, 3), (roll_pitch_sigma, 4)):
        u1 = 1.0 - unit()
        u2 = unit()
        nrm = np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u2)
        if sig > 0.0:
            p[d] += sig * nrm
    return p


def tpe_propose(prior, q, k, trials, xy_range=2.0, yaw_range=np.pi, z_sigma=0.0,
                roll_pitch_sigma=0.0, seed=0):
    """TPE proposal of guided particle k of query q (TreeStructuredParzenEstimator::
    get_next_input, cuda_ndt_matcher/src/tpe.rs:98-196) from the query's aligned results so
    far, rows (x, y, yaw, score) in arrival order: with the results sorted best first (stable),
    the best max(1, min(10, n // 10)) form the good set; the particle's own draw stands unless
    one of 100 further draws (candidate c: the particle stream with the seed xor
    0x94d049bb133111eb * c) has a higher log p_good - 5 log p_bad, where p is a sum of Gaussian
    kernels of 0.25 m, 0.25 m and 2.5 deg on x, y and the wrapped yaw difference."""
    import math
    rows = sorted((tuple(float(v) for v in t) for t in trials), key=lambda t: -t[3])
    n = len(rows)
    above = min(max(n // 10, 1), 10) if n else 0
    kw = dict(xy_range=xy_range, yaw_range=yaw_range, z_sigma=z_sigma,
              roll_pitch_sigma=roll_pitch_sigma)
    pose = particle(prior, q, k, seed=seed, **kw)
    if above == 0:
        return pose
    sig = (0.25, 0.25, 2.5 * math.pi / 180.0)
    lsig = math.log(sig[0]) + math.log(sig[1]) + math.log(sig[2])
    wa = math.log(1.0 / above)
    wb = math.log(1.0 / (n - above)) if n > above else 0.0  # unused when n <= above

    def lse(v):
        if not v:
            return -math.inf
        m = -math.inf
        for x in v:
            m = max(m, x)
        if math.isinf(m):
            return m
        acc = 0.0
        for x in v:
            acc += math.exp(x - m)
        return m + math.log(acc)

    def ratio(c):
        if above >= n:
            return 0.0
        a, b = [], []
        for i, (x, y, yaw, _) in enumerate(rows):
            d = [float(c[0]) - x, float(c[1]) - y, float(c[5]) - yaw]
            while d[2] >= math.pi:
                d[2] -= 2.0 * math.pi
            while d[2] < -math.pi:
                d[2] += 2.0 * math.pi
            lp = 0.0
            for j in range(3):
                r = d[j] / sig[j]
                lp += -0.5 * r * r
            lp -= lsig
            (a if i < above else b).append(lp + (wa if i < above else wb))
        return lse(a) - lse(b) * 5.0

    best = -math.inf
    for c in range(1, 101):
        cand = particle(prior, q, k, seed=seed ^ ((0x94D049BB133111EB * c) & _M64), **kw)
        r = ratio(cand)
        if r > best:
            best = r
            pose = cand
    return pose


def selection_score(nvtl, score):
    """initial_pose.rs:233-245: NVTL when positive, else 5 exp(-score / 10)."""
    return nvtl if nvtl > 0.0 else 5.0 * np.exp(-score / 10.0)


def select_best(results):
    """particle.rs:36-42 (Iterator::max_by: the last of equal maxima)."""
    best, best_sel = -1, -np.inf
    for i, r in enumerate(results):
        sel = selection_score(r["nvtl"], r["score"])
        if best < 0 or sel >= best_sel:
            best, best_sel = i, sel
    return best, best_sel

"""Benchmark: batched NDT scan alignment (20k-point scans against a 5M-point map).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl ours|reference]

One step = one pass of the hot path over one batch of B synthetic 20k-point scans
(128-ring ray-cast lidar on a seeded 400x400 m procedural map of 5M points; initial
guesses from constant-velocity prediction + noise). Prints one JSON line.

- value : aligns/s with the scans already resident in HBM (ndt_align_batch_device),
          CUDA-event time on the library's stream, L2 flushed (256 MB write) between steps.
- e2e   : aligns/s through the public C ABI with host buffers (ndt_align_batch): pinned
          staging, host->device copy of the scans, kernels, device->host copy of results.
- roofline : the Newton kernel's FP32 work (165 FLOP per point-iteration + 65 per
          point-voxel pair, the moment formulation) over its CUDA-event time.
- cpu_baseline : the CPU restatement of the reference's CPU path (NdtOptimizer::align)
          on all host cores, on a bounded sample of the same scans.
--impl reference times that CPU path alone (the reference's own implementation is Rust and
cannot be built here; the restatement stands in for it), and reports beside it the
reference's own GPU kernels (K1-K5, compiled from its sources) driven one alignment at a time
as its host loop drives them ("reference_gpu_kernels").
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "scan aligns/s (20k pts, 5M-pt map); init-pose est/s, learned vs plain"
FLOP_PER_POINT_ITER = 165
FLOP_PER_PAIR = 65
# DRAM bytes (read + write) of one Newton-kernel launch of the default workload (256 scans,
# 5M-point map, seed 2), from one ncu capture of this bench per kernel form
NCU_ALIGN_TRAFFIC = {("k_ndt_align", 256, 5_000_000, 2): 73.3e6,
                     ("k_ndt_queue", 256, 5_000_000, 2): 126.5e6}


def _json_default(o):
    """numpy scalars and arrays in the result line as plain JSON numbers and lists."""
    if isinstance(o, np.generic):
        return o.item()
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(f"{type(o).__name__} is not JSON serialisable")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--map-points", type=int, default=5_000_000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--only", default="",
                    help="comma-separated extra workloads to run instead of all of them "
                         "(init_pose, queue, learned, large_map, large_build, tiles); with "
                         "--steps 0 only those")
    ap.add_argument("--parity", type=int, default=1,
                    help="after timing, check 64 scans of the timed batch against the FP64 "
                         "oracle and the reference's own kernels")
    ap.add_argument("--extras", type=int, default=1,
                    help="also run the initial-pose search and the uneven-queue workloads")
    ap.add_argument("--shape", default="",
                    help="fixed Newton-kernel launch shape "
                         "CLUSTER,THREADS,REGISTERS[,QUEUE[,LANES[,STAGE]]] "
                         "(e.g. 8,256,64 for the cluster kernel, 1,256,64,4 for the work-queue "
                         "kernel with 4 points per thread per chunk, 1,256,64,4,2 with 2 lanes "
                         "per point's neighbour search, 1,256,64,4,1,1 with the chunk's points "
                         "staged in shared memory) instead of the autotuner")
    return ap.parse_args()


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_scan_indices(batch, rank, world):
    """Replicas: every rank aligns its own `batch` scans of the sequence (disjoint shards,
    no collective on the data path); the map is replicated."""
    return [2 + rank * batch + i for i in range(batch)]


def max_over_ranks(values, device):
    """Timing of a multi-rank step: the slowest rank's, reduced on the given device (the
    torch.distributed backend's: cuda for nccl, cpu for gloo)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def make_workload(args, rank, world):
    from cuda_ndt_matcher_gb300 import synth
    n_traj = max(1000, args.batch * world + 8)
    seq = synth.Sequence(seed=args.seed, n_map=args.map_points, n_scans=n_traj)
    ks = rank_scan_indices(args.batch, rank, world)
    scans = [seq.scan(k) for k in ks]
    poses = np.stack([seq.guess(k) for k in ks])
    truth = np.stack([seq.true_pose(k) for k in ks])
    return seq, scans, poses, truth


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_bytes(info):
    """Algorithmic DRAM bytes of one map build as the pipeline runs it (set_target):
    per point: bounds pass (12 B read), key pass (12 B read, key + index written), one
    histogram read and one key+value read and write per 8-bit radix pass over the significant
    key bits (32-bit keys when 3 x max key bits + 1 <= 32, else 64-bit), two key reads for the
    segment starts, and the statistics' index and point gather (16 B); per segment: its start,
    size key and visit order, the two 16-bit size-sort passes, its record (88 B) and validity;
    per voxel: the record read back, the voxel arrays written (104 B), the hash insert's
    reads (64 B) and slot writes (52 B); per slot: the 16 B clear; the dense index: one clear
    and one fill of 16 B per cell; the neighbourhood masks (4 B each, one or eight per cell of
    the grown box): one clear, and one write-back of the words the voxels' atomic ORs set in
    L2."""
    n, S, V, cap = (int(info.num_points), int(info.num_segments), int(info.num_voxels),
                    int(info.hash_capacity))
    lv = max(int(b) for b in info.key_bits)
    end_bit = min(64, 3 * lv + 1)
    kw = 4 if end_bit <= 32 else 8
    passes = (end_bit + 7) // 8
    per_point = 12 + 12 + kw + 4 + passes * (kw + 2 * (kw + 4)) + 2 * kw + 16
    per_seg = 4 + 8 + 2 * 3 * 8 + 88 + 4
    per_vox = 88 + 104 + 64 + 52
    # dense index: the grid (16 B per cell of the box: cleared, then filled) and the
    # neighbourhood masks (the rest of dense_grid_mib: cleared, then written back)
    dense = float(info.dense_grid_mib) * 1024 * 1024
    cells = float(np.prod([int(info.max_coord[a]) - int(info.min_coord[a]) + 1
                           for a in range(3)])) if dense > 0 else 0.0
    grid_bytes = 2 * 16 * cells + 2 * max(dense - 16 * cells, 0.0)
    return int(per_point * n + per_seg * S + per_vox * V + 16 * cap + grid_bytes)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "sm_max_mhz": 2070.0}, "fallback"


def cpu_model():
    """Host CPU model string (lscpu's "Model name", else /proc/cpuinfo's first model field)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model", "hardware")):
                    return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def phase_shares(st):
    keys = ["cycles_points", "cycles_cluster_wait", "cycles_control", "cycles_broadcast"]
    tot = sum(st[k] for k in keys) or 1
    return {k.replace("cycles_", ""): round(st[k] / tot, 4) for k in keys}


def cpu_baseline(grid_args, scans, poses, seconds, semantics="cpu"):
    """Restated reference CPU path on all host cores over a bounded sample of the scans."""
    from oracle import oracle as O
    g = O.Grid(*grid_args)
    cores = os.cpu_count() or 1
    done = 0
    t0 = time.perf_counter()
    i = 0
    while time.perf_counter() - t0 < seconds and i < len(scans):
        j = min(len(scans), i + cores)
        g.align_batch(scans[i:j], poses[i:j], semantics=semantics, nthreads=cores)
        done += j - i
        i = j
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "aligns/s", "cores": cores, "kind": "port",
            "cpu_model": cpu_model(), "nproc": os.cpu_count(),
            "sample": f"{done} of the bench's 20k-point scans, NdtOptimizer::align restated "
                      f"(FP64, all neighbours, ND-clamp + SVD step), {cores} threads, {dt:.1f} s"}


def init_pose_bench(repeats, cpu_seconds):
    """Initial-pose search: 16 queries x 200 particles (x, y +-2 m, yaw over the circle),
    30 iterations, NVTL-ranked, on the 200k-point single-workload map. Wall time of the
    public entry point with host scans (copies, one alignment launch for all 3200
    particles, NVTL scoring, selection), replayed as a CUDA graph."""
    from cuda_ndt_matcher_gb300 import capi, synth
    w = synth.search_queries(seed=21, n_queries=16)
    ctx = capi.Context(cuda_graph=1)
    ctx.set_target(w.map_points)
    kw = dict(num_particles=200, xy_range=2.0, yaw_range=np.pi, seed=5)
    est = ctx.initial_pose_search(w.scans, w.priors, **kw)  # warm-up + graph capture
    ctx.stats_reset()
    t0 = time.perf_counter()
    for r in range(repeats):
        est = ctx.initial_pose_search(w.scans, w.priors, **dict(kw, seed=5 + r))
    wall = time.perf_counter() - t0
    st = ctx.stats()
    ok = 0
    for e, t in zip(est, w.true_poses):
        dyaw = (e["pose"][5] - t[5] + np.pi) % (2 * np.pi) - np.pi
        ok += int(np.linalg.norm(e["pose"][:2] - t[:2]) < 0.2 and abs(dyaw) < np.radians(1.0))
    out = {"metric": "init-pose est/s (plain 200-particle search)",
           "value": 16 * repeats / wall, "unit": "estimates/s", "queries": 16,
           "particles": 200, "ms_per_search_of_16": wall / repeats * 1e3,
           "gpu_ms_per_search_of_16": (st["align_kernel_ms"] + st["score_kernel_ms"]) / repeats,
           "success_rate": ok / len(est), "success": "error < 0.2 m and < 1 deg",
           "scan_points_mean": float(np.mean([len(s) for s in w.scans])), "cuda_graph": True}
    # the reference's own search shape: 200 particles, the last 100 TPE-guided (sequential per
    # query: one launch per guided round for all 16 queries)
    kg = dict(kw, guided=100)
    ctx.initial_pose_search(w.scans, w.priors, **kg)
    t0 = time.perf_counter()
    for r in range(repeats):
        est = ctx.initial_pose_search(w.scans, w.priors, **dict(kg, seed=5 + r))
    wall = time.perf_counter() - t0
    okg = sum(int(_pose_ok(e["pose"], t)) for e, t in zip(est, w.true_poses))
    out["guided"] = {"value": 16 * repeats / wall, "unit": "estimates/s",
                     "ms_per_search_of_16": wall / repeats * 1e3, "particles": 200,
                     "guided_particles": 100, "success_rate": okg / len(est),
                     "launches_per_search": 101}
    ctx.close()
    if cpu_seconds > 0:  # the restated CPU path on the host cores: one query's 200 particles
        from oracle import oracle as O
        g = O.Grid(w.map_points, 2.0)
        cores = os.cpu_count() or 1
        starts = [O.particle(w.priors[0], 0, k, 2.0, np.pi, seed=5) for k in range(200)]
        t0 = time.perf_counter()
        res = g.align_batch([w.scans[0]] * 200, starts, semantics="cpu", nthreads=cores)
        for r in res:
            T = O.pose_T34_zyx(r["pose"])
            g.nvtl(w.scans[0], T)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "estimates/s", "cores": cores,
                               "kind": "port", "sample": f"1 query x 200 particles, "
                               f"NdtOptimizer::align restated + NVTL, {cores} threads, "
                               f"{dt:.1f} s"}
    return out


def _pose_ok(pose, truth):
    dyaw = (pose[5] - truth[5] + np.pi) % (2 * np.pi) - np.pi
    return np.linalg.norm(pose[:2] - truth[:2]) < 0.2 and abs(dyaw) < np.radians(1.0)


def learned_bench(steps=15000, n_maps=50, n_train=400, n_test=200, nvtl_tol=0.01, **net_cfg):
    """Learned initial-pose proposals vs the plain 200-particle search.

    Training: n_maps seeded 200x200 m maps of the sequence generator with n_train scans each;
    labels are plain NDT's converged poses; perturbations x, y U(+-5 m), yaw uniform, drawn on
    the device (steps x train_batch samples, 1024 per step by default). Evaluation: n_test held-out scans per map, coarse poses
    x, y U(+-5 m) with an unknown heading. Plain = 200 particles over the same range;
    learned = 16 proposals refined by NDT; refine8 = then 8 particles (x, y +- 0.5 m, yaw +-
    5 deg) around each query's winner, aligned as a second round; fallback = the plain
    search where the best NVTL is below 2.3 (fallback29: below 2.9).
    - success: error < 0.2 m and < 1 deg against the true pose;
    - judged success (plain NDT as judge): a learned result counts only if it succeeds and
      its converged NVTL matches the plain search's on the same query (within nvtl_tol
      relative, or higher);
    - GPU time per query: the Newton and scoring kernels plus, for the learned searches, the
      proposal network's device work (features, GEMMs, decode), all CUDA-event timed."""
    from cuda_ndt_matcher_gb300 import capi, synth
    t0 = time.perf_counter()
    maps = synth.proposal_maps(seed=100, n_maps=n_maps, n_train=n_train, n_test=n_test)
    net = capi.PNet(seed=7, **net_cfg)
    ctx = capi.Context(cuda_graph=1)
    mids = []
    for m in maps:
        mid = net.add_map(m.map_points)
        mids.append(mid)
        ctx.set_target(m.map_points)
        for s, r in zip(m.train_scans, ctx.align_batch(m.train_scans, m.train_poses)):
            net.add_scan(mid, s, r["pose"])
    prep = time.perf_counter() - t0
    import torch
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net.train(steps - 200, record_loss=False)
    loss = net.train(200)
    train_s = time.perf_counter() - t1
    nst = net.stats()
    cfg = net.cfg
    dims = [cfg.input_dim] + [cfg.hidden] * cfg.hidden_layers + [4 * cfg.proposals]
    pairs = list(zip(dims[:-1], dims[1:]))
    flops_step = 2 * cfg.train_batch * (2 * sum(i * o for i, o in pairs) + sum(i * o for i, o in pairs[1:]))
    rng = np.random.default_rng(99)
    names = ("plain_200", "learned_16", "learned_16_refine8", "learned_16_refine8_fallback",
             "learned_16_refine8_fallback29")
    out = {k: {"ok": 0, "judged": 0, "nvtl_match": 0, "gpu_ms": 0.0, "net_ms": 0.0,
               "wall_s": 0.0, "fallbacks": 0} for k in names}
    n = 0
    for m, mid in zip(maps, mids):
        ctx.set_target(m.map_points)
        coarse = []
        for t in m.test_poses:
            c = t.copy()
            c[:2] += rng.uniform(-5, 5, 2)
            c[5] = rng.uniform(-np.pi, np.pi)
            coarse.append(c)
        fb = []
        plain_cfg = dict(num_particles=200, xy_range=5.0, yaw_range=np.pi, seed=3)
        refine = dict(num_particles=8, xy_range=0.5, yaw_range=np.radians(5.0), seed=5)
        runs = {
            "plain_200": lambda: ctx.initial_pose_search(m.test_scans, coarse, **plain_cfg),
            "learned_16": lambda: ctx.learned_pose_search(net, mid, m.test_scans, coarse),
            "learned_16_refine8": lambda: ctx.learned_pose_search(
                net, mid, m.test_scans, coarse, refine=refine),
            "learned_16_refine8_fallback": lambda: ctx.learned_pose_search(
                net, mid, m.test_scans, coarse, refine=refine, nvtl_threshold=2.3,
                fallback=plain_cfg),
            "learned_16_refine8_fallback29": lambda: ctx.learned_pose_search(
                net, mid, m.test_scans, coarse, refine=refine, nvtl_threshold=2.9,
                fallback=plain_cfg)}
        plain = None
        for name in names:
            ctx.stats_reset()
            ts = time.perf_counter()
            est = runs[name]()
            out[name]["wall_s"] += time.perf_counter() - ts
            st = ctx.stats()
            out[name]["gpu_ms"] += (st["align_kernel_ms"] + st["score_kernel_ms"] +
                                    st["proposal_kernel_ms"])
            out[name]["net_ms"] += st["proposal_kernel_ms"]
            if plain is None:
                plain = est
            for e, p, t in zip(est, plain, m.test_poses):
                ok = bool(_pose_ok(e["pose"], t))
                match = e["nvtl"] >= p["nvtl"] - nvtl_tol * abs(p["nvtl"])
                out[name]["ok"] += ok
                out[name]["nvtl_match"] += bool(match)
                out[name]["judged"] += ok and bool(match)
            out[name]["fallbacks"] += sum(int(e.get("fallback", False)) for e in est)
        n += len(m.test_poses)
    res = {"metric": "init-pose est/s, learned vs plain", "queries": n,
           "training": {"maps": len(maps), "scans": sum(len(m.train_scans) for m in maps),
                        "steps": steps, "batch": cfg.train_batch, "samples": steps * cfg.train_batch,
                        "seconds": train_s,
                        "device_ms": nst["train_ms"], "prep_seconds": prep,
                        "final_loss": float(loss.mean()),
                        "roofline": {"bound": "tensor", "kernel": "k_gemm_bf16_tn (training step)",
                                     "achieved": flops_step * steps / (nst["train_ms"] / 1e3) / 1e12,
                                     "peak": peaks()[0].get("bf16_tflops_sustained"),
                                     "unit": "TFLOP/s",
                                     "note": "GEMM FLOPs of whole training steps over their "
                                             "CUDA-event time (sampling, features, elementwise "
                                             "and Adam included)"}},
           "judge": f"learned success counts only if its NVTL >= the plain search's NVTL - "
                    f"{nvtl_tol:g} x |NVTL| on the same query",
           "gpu_time": "Newton + scoring kernels + proposal network (features, GEMMs, decode), "
                       "CUDA events"}
    for name, r in out.items():
        res[name] = {"success_rate": r["ok"] / n, "judged_success_rate": r["judged"] / n,
                     "nvtl_matches_plain": r["nvtl_match"] / n,
                     "gpu_ms_per_query": r["gpu_ms"] / n,
                     "network_ms_per_query": r["net_ms"] / n,
                     "est_per_s": n / r["wall_s"], "fallback_rate": r["fallbacks"] / n}
    pk = res["training"]["roofline"]["peak"]
    if pk:
        res["training"]["roofline"]["frac"] = res["training"]["roofline"]["achieved"] / pk
    for name in names[1:]:
        res[name]["gpu_time_ratio_plain_over_this"] = (
            res["plain_200"]["gpu_ms_per_query"] / max(res[name]["gpu_ms_per_query"], 1e-9))
    net.close()
    ctx.close()
    return res


def tile_stream_bench(pts, scans, guesses, events=40):
    """Tiles of 100 x 100 m streamed over the large map at 2 m: a 5 x 5 tile window slides
    east one tile column at a time. Each event puts one tile (upload + its cells' statistics),
    drops the one leaving the window and commits a background merge of the resident tiles'
    cells, while a batch of dense scans is aligned on the current map. Reported: device time
    per event (the put's cell statistics + the merge), wall time per event (upload, put,
    commit, aligning the batch, waiting for the merge) and the tile rate that wall time
    sustains."""
    from cuda_ndt_matcher_gb300 import capi
    tx = np.floor(pts[:, 0] / 100.0).astype(np.int64)
    ty = np.floor(pts[:, 1] / 100.0).astype(np.int64)
    tid = (tx + 10) * 32 + (ty + 10)
    order = np.argsort(tid, kind="stable")
    bounds = np.searchsorted(tid[order], np.arange(32 * 32 + 1))
    tile = lambda i, j: pts[order[bounds[(i + 10) * 32 + (j + 10)]:bounds[(i + 10) * 32 + (j + 10) + 1]]]
    ctx = capi.Context(resolution=2.0, cuda_graph=1)
    window = [(i, j) for i in range(-7, -2) for j in range(-2, 3)]
    for (i, j) in window:
        ctx.tile_put((i + 10) * 32 + (j + 10), tile(i, j))
    ctx.tiles_commit(wait=True)
    ev = [(i, j) for i in range(-2, -2 + events // 5 + 1) for j in range(-2, 3)][:events]
    build_ms, put_ms, wall = [], [], []
    for k, (i, j) in enumerate(ev):
        t0 = time.perf_counter()
        ctx.tile_put((i + 10) * 32 + (j + 10), tile(i, j))
        put_ms.append(ctx.tiles_status()["put_ms"])
        old = (i - 5, j)
        ctx.tile_remove((old[0] + 10) * 32 + (old[1] + 10))
        ctx.tiles_commit(wait=False)
        ctx.align_batch(scans, guesses)        # alignment continues on the current map
        while ctx.tiles_status()["pending"]:
            time.sleep(0.0002)
        ctx.map_info()                         # switch to the merged map
        wall.append(time.perf_counter() - t0)
        build_ms.append(ctx.tiles_status()["build_ms"])
    st = ctx.tiles_status()
    # the same window rebuilt from all its points at once, for comparison
    full = capi.Context(resolution=2.0)
    win = np.concatenate([tile(i, j) for (i, j) in ev[-25:]])
    full.set_target(win)
    full.set_target(win)
    full_ms = float(full.map_info().build_ms)
    full.close()
    ctx.close()
    return {"tile_m": 100, "window_tiles": 25, "points_in_window": int(st["points"]),
            "events": len(ev), "put_cell_stats_ms_mean": float(np.mean(put_ms)),
            "merge_ms_mean": float(np.mean(build_ms)), "merge_ms_max": float(np.max(build_ms)),
            "device_ms_per_event": float(np.mean(put_ms) + np.mean(build_ms)),
            "full_window_rebuild_ms": full_ms,
            "event_wall_ms_mean": float(np.mean(wall) * 1e3),
            "sustained_tiles_per_s": float(1.0 / np.mean(wall)),
            "aligned_per_event": len(scans)}


def large_map_bench(n_points=50_000_000, n_scans=16):
    """Large-map stress: 50M points over 2 x 2 km (sequence generator densities, 5% uniform
    outliers) built at 1, 2 and 3 m. Per resolution:
    - build time (CUDA events around the build) and GB/s of the pipeline's bytes
      (build_bytes);
    - hash load factor;
    - 20 sampled voxels against the oracle's build of exactly that cell's points: coordinates,
      counts and FP64 means bit for bit, covariance and inverse in f32 ULP of the matrix scale;
    - the largest FP32-vs-FP64 covariance difference over the samples. The FP32 value is the
      reference GPU pipeline's cell-centre-shifted single-precision formula; the FP64 value
      is the library's.
    It then aligns 16 dense 100k-point crop scans and reports aligns/s."""
    from cuda_ndt_matcher_gb300 import capi, synth
    from oracle import oracle as O
    pts = synth.large_map(seed=7, extent=2000.0, n_points=n_points)
    rng = np.random.default_rng(11)
    poses, scans, guesses = [], [], []
    inner = pts[(np.abs(pts[:, 0]) < 900) & (np.abs(pts[:, 1]) < 900)]
    for i in range(n_scans):
        p = np.array([rng.uniform(-800, 800), rng.uniform(-800, 800), 1.8, 0, 0,
                      rng.uniform(-np.pi, np.pi)])
        near = inner[(np.abs(inner[:, 0] - p[0]) < 61) & (np.abs(inner[:, 1] - p[1]) < 61)]
        scans.append(synth.crop_scan(near, p, 100_000, seed=i))
        g = p.copy()
        g[:2] += rng.uniform(-0.3, 0.3, 2)
        g[5] += np.radians(rng.uniform(-1.0, 1.0))
        poses.append(p)
        guesses.append(g)
    out = {"points": int(len(pts)), "extent_m": 2000, "outliers": 0.05, "resolutions": {}}
    for res in (1.0, 2.0, 3.0):
        ctx = capi.Context(resolution=res, cuda_graph=1)
        ctx.set_target(pts)                # allocations
        ctx.set_target(pts)                # timed rebuild
        info = ctx.map_info()
        nbytes = build_bytes(info)
        coords, means, covs, icovs, counts = ctx.map_voxels()
        pick = rng.choice(len(coords), 20, replace=False)
        exact, fp32_err, cov_ulp, icov_ulp = True, 0.0, 0.0, 0.0
        for v in pick:
            c = coords[v]
            lo = c.astype(np.float32) * np.float32(res)
            m = np.all((pts >= lo - np.float32(res) * 0.001) &
                       (pts < lo + np.float32(res) * 1.001), axis=1)
            members = pts[m]
            members = members[np.all(np.floor(members / np.float32(res)).astype(np.int64)
                                     == c, axis=1)]
            g = O.Grid(members, res, centered=True)
            exact &= bool(g.n == 1 and np.array_equal(g.coords[0], c) and
                          g.counts[0] == counts[v] and np.array_equal(g.means[0], means[v]))
            if g.n == 1:
                cov_ulp = max(cov_ulp, _matrix_ulps(g.covs[0], covs[v]))
                icov_ulp = max(icov_ulp, _matrix_ulps(g.icovs[0], icovs[v]))
            ctr = (lo + np.float32(res / 2)).astype(np.float32)
            q = (members - ctr).astype(np.float32)
            mu = np.float32(0) + q.sum(0, dtype=np.float32) / np.float32(len(q))
            d = (q - mu).astype(np.float32)
            c32 = (d.T.astype(np.float32) @ d.astype(np.float32)) / np.float32(len(q) - 1)
            c64 = covs[v].reshape(3, 3).astype(np.float64)
            fp32_err = max(fp32_err, float(np.abs(c32 - c64).max() / max(np.abs(c64).max(), 1e-30)))
        ctx.stats_reset()
        t0 = time.perf_counter()
        res_al = ctx.align_batch(scans, guesses)
        wall = time.perf_counter() - t0
        st = ctx.stats()
        err = [float(np.linalg.norm(r["pose"][:2] - p[:2])) for r, p in zip(res_al, poses)]
        if res == 2.0:
            out["tile_streaming"] = tile_stream_bench(pts, scans, guesses)
        out["resolutions"][f"{res:g}m"] = {
            "voxels": int(info.num_voxels), "build_ms": float(info.build_ms),
            "build_gbs": nbytes / (info.build_ms / 1e3) / 1e9,
            "build_hbm_frac": nbytes / (info.build_ms / 1e3) / 1e9 / peaks()[0]["hbm_gbs"],
            "hash_capacity": int(info.hash_capacity),
            "hash_load": info.num_voxels / info.hash_capacity, "max_probe": int(info.max_probe),
            "cell_index": (f"dense grid {info.dense_grid_mib:.0f} MiB, "
                           f"{info.masks_per_cell} mask(s) per cell"
                           if info.dense_grid_mib > 0 else "hash"),
            "sampled_voxels_membership_counts_means_bitexact_vs_oracle": exact,
            "sampled_cov_max_f32_ulp": cov_ulp, "sampled_icov_max_f32_ulp": icov_ulp,
            "sampled": len(pick),
            "fp32_vs_fp64_cov_rel_err_max": fp32_err,
            "dense_scan_aligns_per_s": len(scans) / (st["align_kernel_ms"] / 1e3),
            "dense_scan_iterations_per_align": st["iterations"] / max(st["alignments"], 1),
            "dense_scan_pairs_per_point_iter": st["correspondences"] /
            max(st["point_iterations"], 1),
            "dense_scan_kernel_us_per_point_iter": st["align_kernel_ms"] * 1e3 /
            max(st["point_iterations"], 1),
            "dense_scan_e2e_aligns_per_s": len(scans) / wall,
            "dense_scan_median_err_m": float(np.median(err))}
        if res == 2.0:
            res_2m = res_al
        ctx.close()
    # the 2 m map with a neighbourhood mask per octant of each cell (NDT_CELL_INDEX_OCTANT;
    # the automatic choice keeps one mask per cell at this size): build and the same scans
    ctx = capi.Context(resolution=2.0, cuda_graph=1, cell_index=2)
    ctx.set_target(pts)
    ctx.set_target(pts)
    info = ctx.map_info()
    ctx.stats_reset()                      # timed as the resolutions above
    res_oct = ctx.align_batch(scans, guesses)
    st = ctx.stats()
    out["2m_octant_masks"] = {
        "build_ms": float(info.build_ms),
        "cell_index": f"dense grid {info.dense_grid_mib:.0f} MiB, {info.masks_per_cell} "
                      f"mask(s) per cell",
        "dense_scan_aligns_per_s": len(scans) / (st["align_kernel_ms"] / 1e3),
        "same_results_as_2m": bool(all(np.array_equal(a["pose"], b["pose"]) and
                                       a["iterations"] == b["iterations"]
                                       for a, b in zip(res_oct, res_2m)))}
    ctx.close()
    return out


def large_build_bench(n_points=50_000_000, repeats=3):
    """The large map's builds alone: the 50M-point 2 x 2 km map set as the target at 1, 2 and
    3 m, one untimed build (allocations) then `repeats` builds, CUDA-event time of each; bytes
    by build_bytes."""
    from cuda_ndt_matcher_gb300 import capi, synth
    pts = synth.large_map(seed=7, extent=2000.0, n_points=n_points)
    out = {}
    for res in (1.0, 2.0, 3.0):
        ctx = capi.Context(resolution=res)
        ctx.set_target(pts)
        ms = []
        for _ in range(repeats):
            ctx.set_target(pts)
            ms.append(float(ctx.map_info().build_ms))
        info = ctx.map_info()
        b = build_bytes(info)
        out[f"{res:g}m"] = {"voxels": int(info.num_voxels), "segments": int(info.num_segments),
                            "build_ms": min(ms), "bytes": b,
                            "build_gbs": b / (min(ms) / 1e3) / 1e9,
                            "build_hbm_frac": b / (min(ms) / 1e3) / 1e9 / peaks()[0]["hbm_gbs"]}
        ctx.close()
    return out


def parity_sample(seq_map, scans, poses, results, n=64):
    """Checker run after the timed regions: the first n scans of the timed batch, as the last
    timed step aligned them, against the FP64 oracle (graph semantics, the same inputs) and
    against the reference's own graph kernels K1-K5 (compiled from its sources, one alignment
    at a time). Reports max and p99 of the pose, score and NVTL differences to FP64, the
    scans meeting the per-scan bar (iterations equal, 1e-4 m, 1e-5 rad, 1e-5 relative), and
    how often this library and the FP64 oracle each agree with the reference."""
    from oracle import oracle as O
    n = min(n, len(scans))
    g = O.Grid(seq_map, 2.0)
    want = g.align_batch(scans[:n], poses[:n], semantics="gpu")
    got = results[:n]
    dpos = np.array([np.abs(a["pose"][:3] - b["pose"][:3]).max() for a, b in zip(got, want)])
    drot = np.array([np.abs(a["pose"][3:] - b["pose"][3:]).max() for a, b in zip(got, want)])
    rel = lambda k: np.array([abs(a[k] - b[k]) / max(abs(b[k]), 1e-30)
                              for a, b in zip(got, want)])
    dsc, dnv = rel("score"), rel("nvtl")
    same_it = np.array([a["iterations"] == b["iterations"] for a, b in zip(got, want)])
    bar = same_it & (dpos <= 1e-4) & (drot <= 1e-5) & (dsc <= 1e-5) & (dnv <= 1e-5)
    q = lambda v: {"max": float(v.max()), "p99": float(np.percentile(v, 99)),
                   "median": float(np.median(v))}
    # the oracle's own sensitivity: scans whose FP64 trajectory from a start moved by 1e-7
    # (x, y or yaw) misses the same bar against the unmoved one
    sensitive = set()
    for axis in (0, 1, 5):
        p2 = np.array(poses[:n], np.float64).copy()
        p2[:, axis] += 1e-7
        for i, (a, b) in enumerate(zip(g.align_batch(scans[:n], p2, semantics="gpu"), want)):
            if not (a["iterations"] == b["iterations"]
                    and np.abs(a["pose"][:3] - b["pose"][:3]).max() <= 1e-4
                    and np.abs(a["pose"][3:] - b["pose"][3:]).max() <= 1e-5):
                sensitive.add(i)
    out = {"scans": n, "against": "FP64 oracle, graph semantics (or_align_gpu_sem)",
           "oracle_self_sensitive_ids": sorted(sensitive),
           "pose_m": q(dpos), "pose_rad": q(drot), "score_rel": q(dsc), "nvtl_rel": q(dnv),
           "iterations_equal": int(same_it.sum()), "within_bar": int(bar.sum()),
           "outside_bar_ids": [int(i) for i in np.nonzero(~bar)[0]]}
    try:
        from oracle import ref_graph
        if not ref_graph.available():
            raise RuntimeError("reference cubins not built")
        rg = ref_graph.RefGraph()
        rg.set_map(g.means, g.icovs, 2.0)
        d1, d2 = (float(np.float32(x)) for x in O.gauss_params(2.0, 0.55))
        same = lambda a, b: (a["iterations"] == b["iterations"]
                             and np.abs(a["pose"][:3] - b["pose"][:3]).max() <= 1e-4
                             and np.abs(a["pose"][3:] - b["pose"][3:]).max() <= 1e-5)
        ours = fp64 = 0
        for k in range(n):
            r = rg.align(scans[k], poses[k], d1, d2)
            ours += same(got[k], r)
            fp64 += same(want[k], r)
        rg.close()
        out["reference_k1_k5_agreement"] = {"ours": ours, "fp64_oracle": fp64, "of": n,
                                            "rule": "iterations equal, 1e-4 m, 1e-5 rad"}
    except Exception as e:
        out["reference_k1_k5_agreement"] = {"unavailable": f"{type(e).__name__}: {e}"}
    return out


def _matrix_ulps(a, b):
    """Largest entry difference of two 3x3 matrices in f32 spacings at their scale."""
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    scale = np.float32(max(np.abs(a).max(), np.abs(b).max()))
    return float(np.abs(a - b).max() / max(float(np.spacing(scale)), 1e-45))


def queue_bench(repeats):
    """A queue of 64 scans of log-uniform size 2k-40k points in one launch (CUDA graph):
    throughput and per-scan completion latency (device clock, from the batch's first start)."""
    from cuda_ndt_matcher_gb300 import capi, synth
    w = synth.queue_scans(seed=22, n_scans=64)
    ctx = capi.Context(cuda_graph=1)
    ctx.set_target(w.map_points)
    ctx.align_batch(w.scans, w.priors)
    lat = []
    t0 = time.perf_counter()
    for _ in range(repeats):
        ctx.align_batch(w.scans, w.priors)
        _, fin = ctx.batch_timings(len(w.scans))
        lat.append(fin)
    wall = time.perf_counter() - t0
    lat = np.concatenate(lat)
    out = {"metric": "queue aligns/s (64 scans, 2k-40k points, one launch)",
           "value": 64 * repeats / wall, "unit": "aligns/s",
           "latency_ms_p50": float(np.percentile(lat, 50)),
           "latency_ms_p99": float(np.percentile(lat, 99)),
           "latency": "scan completion on the device clock from the batch's first start",
           "points": [int(min(len(s) for s in w.scans)), int(max(len(s) for s in w.scans))],
           "cuda_graph": True}
    ctx.close()
    return out


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    seq, scans, poses, _ = make_workload(args, 0, 1)
    from oracle import oracle as O
    g = O.Grid(seq.map, 2.0)
    cores = os.cpu_count() or 1
    per_step = cores
    times = []
    for s in range(args.warmup + args.steps):
        i0 = (s * per_step) % max(1, len(scans) - per_step)
        t0 = time.perf_counter()
        g.align_batch(scans[i0:i0 + per_step], poses[i0:i0 + per_step], semantics="cpu",
                      nthreads=cores)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = per_step * args.steps / total
    ref_gpu = reference_gpu_kernels(g, scans, poses)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "aligns/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sequence: 5M-pt 400x400 m map, 20k-pt 128-ring scans, "
                               "batched alignment", "batch": args.batch, "scan_points": 20000,
                   "map_points": args.map_points, "semantics": "CPU path (NDT_USE_GPU=0)",
                   "sampled_scans_per_step": per_step,
                   "sample_rule": f"each step aligns {per_step} scans of the {args.batch}-scan "
                                  "batch (one per host thread); aligns/s is per alignment, so "
                                  "the rate compares with the GPU arm's"},
        "cpu_baseline": {"value": value, "unit": "aligns/s", "cores": cores, "kind": "port",
                         "cpu_model": cpu_model(), "nproc": os.cpu_count(),
                         "sample": f"{per_step} scans per step, NdtOptimizer::align restated "
                                   "(the Rust reference cannot be built here)"},
        "e2e": {"value": value, "unit": "aligns/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_gpu_kernels": ref_gpu,
    }
    print(json.dumps(line, default=_json_default), flush=True)


def reference_gpu_kernels(grid, scans, poses, n=64):
    """The reference's own GPU path for comparison: its graph kernels K1-K5 and voxel hash
    (src/cuda_ffi/csrc, compiled unmodified into sm_103a cubins) driven one alignment at a
    time by the restated FullGpuPipelineV2::optimize loop, on the first n scans of the
    workload. The map upload and hash build happen once, before timing (the reference
    repeats them on every align call)."""
    try:
        from oracle import oracle as O, ref_graph
        if not ref_graph.available():
            return {"unavailable": "reference cubins not built"}
        rg = ref_graph.RefGraph()
        rg.set_map(grid.means, grid.icovs, 2.0)
        d1, d2 = (float(np.float32(x)) for x in O.gauss_params(2.0, 0.55))
        n = min(n, len(scans))
        for k in range(2):  # module load, first allocations
            rg.align(scans[k], poses[k], d1, d2)
        t0 = time.perf_counter()
        iters = 0
        for k in range(n):
            iters += rg.align(scans[k], poses[k], d1, d2)["iterations"]
        dt = time.perf_counter() - t0
        rg.close()
        return {"value": n / dt, "unit": "aligns/s", "ms_per_align": 1000 * dt / n,
                "iterations_per_align": iters / n,
                "sample": f"{n} of the workload's scans, one align call each: K1, then K2/K3/K5 "
                          "per iteration with a device sync and a flag read (the reference's "
                          "host loop), points uploaded per call; voxels of the oracle's build"}
    except Exception as e:  # no device, or the driver library could not load
        return {"unavailable": f"{type(e).__name__}: {e}"}


def run_ours(args):
    import torch
    from cuda_ndt_matcher_gb300 import capi

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seq, scans, poses, truth = make_workload(args, rank, world)
    ctx = capi.Context(device=local)
    ctx.set_target(seq.map)      # first build: allocations
    ctx.set_target(seq.map)      # the reported build
    info = ctx.map_info()
    build_ms = float(info.build_ms)

    # device-resident inputs
    counts = np.array([len(s) for s in scans], np.uint64)
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    allpts = np.concatenate(scans).astype(np.float32)
    d_pts = torch.from_numpy(allpts).cuda()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB
    stream = torch.cuda.ExternalStream(ctx.stream)
    import ctypes as C
    off_c = np.ascontiguousarray(offsets)
    pose_c = np.ascontiguousarray(poses, np.float64)
    B = len(scans)
    res_arr = (capi.Result * B)()

    def step_device():
        capi.check(ctx.lib.ndt_align_batch_device(ctx.h, C.c_void_p(d_pts.data_ptr()),
                                                  off_c.ctypes.data, pose_c.ctypes.data, B,
                                                  res_arr))

    scan_arr = (capi.Scan * B)()
    for i, s in enumerate(scans):
        scan_arr[i].xyz = s.ctypes.data
        scan_arr[i].num_points = len(s)
        for k in range(6):
            scan_arr[i].initial_pose[k] = float(poses[i][k])
    res_e2e = (capi.Result * B)()

    def step_host():
        capi.check(ctx.lib.ndt_align_batch(ctx.h, scan_arr, B, res_e2e))

    if args.shape:
        vals = [int(v) for v in args.shape.split(",")]
        K, T, R = vals[:3]
        Q = vals[3] if len(vals) > 3 else 0
        L = vals[4] if len(vals) > 4 else 1
        St = vals[5] if len(vals) > 5 else 0
        ctx.configure(cluster_size=K, threads_per_cta=T, max_registers=R,
                      work_queue=Q if Q > 0 else -1, lanes_per_point=L if Q > 0 else 0,
                      stage_points=St if Q > 0 else 0)
        tune = {"cluster_size": K, "threads_per_cta": T, "registers": R, "work_queue": Q,
                "lanes_per_point": L if Q > 0 else 0, "stage_points": St if Q > 0 else 0,
                "chosen_by": "--shape"}
    else:
        # launch shape for this batch class, chosen by the library's autotuner (untimed)
        tune = ctx.autotune(C.c_void_p(d_pts.data_ptr()), off_c, pose_c, repeats=1)
        tune["chosen_by"] = "ndt_autotune"
    for _ in range(args.warmup):
        step_device()
        step_host()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    # timed region 1: device-resident value (CUDA events on the library stream)
    ctx.stats_reset()
    clocks = ClockSampler(local)
    clocks.start()
    evs = []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_device()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    st = ctx.stats()
    # timed region 2: end to end through the host-buffer C ABI
    ctx.stats_reset()
    wall = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        step_host()
        torch.cuda.synchronize()
        wall += time.perf_counter() - t1
    st_e2e = ctx.stats()
    # timed region 3: the same batches as a stream through the asynchronous C ABI
    # (ndt_batch_submit / ndt_batch_wait, two batches in flight): one batch's staging and
    # copies, and the start of its kernels, overlap the previous batch's kernels
    res_stream = [(capi.Result * B)() for _ in range(2)]
    for k in range(max(args.warmup, 2)):  # every slot staged once (buffers, pinned memory)
        tk = C.c_uint64()
        capi.check(ctx.lib.ndt_batch_submit(ctx.h, scan_arr, B, C.byref(tk)))
        if k % 2:
            capi.check(ctx.lib.ndt_batch_wait(ctx.h, prev, res_stream[0]))
            capi.check(ctx.lib.ndt_batch_wait(ctx.h, tk.value, res_stream[1]))
        prev = tk.value
    if max(args.warmup, 2) % 2:
        capi.check(ctx.lib.ndt_batch_wait(ctx.h, prev, res_stream[0]))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    pending = []
    for k in range(args.steps):
        if len(pending) == 2:
            tk, buf = pending.pop(0)
            capi.check(ctx.lib.ndt_batch_wait(ctx.h, tk, buf))
        tk = C.c_uint64()
        capi.check(ctx.lib.ndt_batch_submit(ctx.h, scan_arr, B, C.byref(tk)))
        pending.append((tk.value, res_stream[k % 2]))
    for tk, buf in pending:
        capi.check(ctx.lib.ndt_batch_wait(ctx.h, tk, buf))
    wall_stream = time.perf_counter() - t1
    clk = clocks.stop()
    if world > 1:
        dev_ms, wall, wall_stream = max_over_ranks([dev_ms, wall, wall_stream], "cuda")

    aligns = B * args.steps * world
    value = aligns / (dev_ms / 1000.0)
    e2e = aligns / wall
    e2e_stream = aligns / wall_stream
    pk, src = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    flops = FLOP_PER_POINT_ITER * st["point_iterations"] + FLOP_PER_PAIR * st["correspondences"]
    kern_s = st["align_kernel_ms"] / 1000.0
    achieved = flops / kern_s / 1e12 if kern_s > 0 else 0.0
    launches = st["align_launches"]
    # accuracy of this run against the true poses (diagnostic)
    got = np.array([list(r.pose) for r in res_arr])
    perr = np.linalg.norm(got[:, :2] - truth[:, :2], axis=1)
    bbytes = build_bytes(info)

    parity = None
    if rank == 0 and args.parity:
        parity = parity_sample(seq.map, scans, poses,
                               [capi.result_dict(r) for r in res_arr], n=64)
    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        cpu = cpu_baseline((seq.map, 2.0), scans, poses, args.cpu_seconds)
    extra = {}
    if rank == 0 and args.extras:
        for key, fn in (("init_pose", lambda: init_pose_bench(5, args.cpu_seconds)),
                        ("queue", lambda: queue_bench(10)),
                        ("learned_init_pose", learned_bench),
                        ("large_map", large_map_bench)):
            try:
                extra[key] = fn()
            except Exception as e:  # one workload's failure must not lose the headline line
                extra[key] = {"error": f"{type(e).__name__}: {e}"}
    elif rank == 0 and args.only:
        extra = run_only(args.only, args)
    kname = "k_ndt_queue" if tune["work_queue"] else "k_ndt_align"
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "aligns/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 reductions and 6x6 solve)",
            "data": "synthetic",
            "config": {"workload": "sequence: 5M-pt 400x400 m map, 20k-pt 128-ring scans, "
                                   "batched alignment", "batch": B, "scan_points": 20000,
                       "map_points": args.map_points, "map_voxels": int(info.num_voxels),
                       "cell_index": (f"dense grid {info.dense_grid_mib:.1f} MiB, "
                                      f"{info.masks_per_cell} neighbourhood mask(s) per cell"
                                      if info.dense_grid_mib > 0 else "hash"),
                       "semantics": "graph kernels K1-K5", "l2": "flushed (256 MB write) "
                       "between steps",
                       "launch_shape": {"cluster_size": tune["cluster_size"],
                                        "threads_per_cta": tune["threads_per_cta"],
                                        "registers": tune["registers"],
                                        "work_queue_points_per_thread": tune["work_queue"],
                                        "lanes_per_point": tune.get("lanes_per_point", 0),
                                        "stage_points": tune.get("stage_points", 0),
                                        "chosen_by": tune["chosen_by"]}},
            "e2e": {"value": e2e, "unit": "aligns/s",
                    "h2d_bytes_per_step": int(st_e2e["h2d_bytes"] // max(args.steps, 1)),
                    "d2h_bytes_per_step": int(st_e2e["d2h_bytes"] // max(args.steps, 1)),
                    "call": "ndt_align_batch (one synchronous batch per step)"},
            "e2e_stream": {"value": e2e_stream, "unit": "aligns/s",
                           "call": "ndt_batch_submit / ndt_batch_wait, two batches in flight",
                           "batches": args.steps},
            "roofline": {"bound": "fp32", "kernel": kname, "achieved": achieved,
                         "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None,
                         "traffic": NCU_ALIGN_TRAFFIC.get((kname, B, args.map_points, args.seed)),
                         "traffic_unit": "bytes per launch (ncu dram read + write)",
                         "peak_source": f"derived: SMs x 128 FP32 lanes x 2 x sm_max_mhz "
                                        f"({src} MEASURED_PEAKS.json clock)",
                         "flops_per_launch": flops / max(launches, 1),
                         "avg_launch_ms": st["align_kernel_ms"] / max(launches, 1),
                         "iterations_per_align": st["iterations"] / max(st["alignments"], 1),
                         "pairs_per_point_iter": st["correspondences"] /
                         max(st["point_iterations"], 1),
                         "phase_cycles_share": phase_shares(st),
                         "eigen_solves_per_align": st["eigen_solves"] /
                         max(st["alignments"], 1)},
            "build_roofline": {"bound": "hbm", "achieved": bbytes / (build_ms / 1e3) / 1e9,
                               "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                               "frac": bbytes / (build_ms / 1e3) / 1e9 / pk.get("hbm_gbs"),
                               "build_ms": build_ms, "bytes": int(bbytes),
                               "bytes_rule": "bench.build_bytes: the pipeline's passes as run",
                               "peak_source": src},
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clk,
            "gpu_launches": int(st["align_launches"] + 2 * st["score_launches"]),
            "accuracy": {"median_xy_err_m": float(np.median(perr)),
                         "p99_xy_err_m": float(np.percentile(perr, 99))},
        }
        line.update(extra)
        print(json.dumps(line, default=_json_default), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_only(names, args):
    """The named extra workloads alone (comma-separated: init_pose, queue, learned,
    large_map, large_build, tiles)."""
    out = {}
    for nm in names.split(","):
        if nm == "init_pose":
            out["init_pose"] = init_pose_bench(5, args.cpu_seconds)
        elif nm == "queue":
            out["queue"] = queue_bench(10)
        elif nm == "learned":
            out["learned_init_pose"] = learned_bench()
        elif nm == "large_map":
            out["large_map"] = large_map_bench()
        elif nm == "large_build":
            out["large_build"] = large_build_bench()
        elif nm == "tiles":
            from cuda_ndt_matcher_gb300 import synth
            pts = synth.large_map(seed=7, extent=2000.0, n_points=50_000_000)
            rng = np.random.default_rng(11)
            scans, guesses = [], []
            for i in range(16):
                p = np.array([rng.uniform(-800, 800), rng.uniform(-800, 800), 1.8, 0, 0,
                              rng.uniform(-np.pi, np.pi)])
                near = pts[(np.abs(pts[:, 0] - p[0]) < 61) & (np.abs(pts[:, 1] - p[1]) < 61)]
                scans.append(synth.crop_scan(near, p, 100_000, seed=i))
                guesses.append(p)
            out["tile_streaming"] = tile_stream_bench(pts, scans, guesses)
        else:
            raise SystemExit(f"unknown workload {nm}")
    return out


def main():
    args = parse()
    if args.only and args.impl == "ours" and args.steps == 0:
        print(json.dumps(run_only(args.only, args), default=_json_default), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

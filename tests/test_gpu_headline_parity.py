"""Per-scan parity on the headline workload, through the C ABI.

Workload: the seeded 5M-point 400 x 400 m sequence map (seed 2, 138k voxels at 2 m) and 64
of its 128-ring scans subsampled to 20,000 points (sequence indices 2..65, the first 64 scans
of the benchmark's batch), each started from its constant-velocity guess. All 64 are aligned
in ONE batch with the Newton-kernel launch shape the autotuner picks for that batch, as the
benchmark aligns them.

Bar, per scan, against the FP64 oracle's graph semantics (or_align_gpu_sem, the restatement of
FullGpuPipelineV2::optimize, src/ndt_cuda/src/optimization/full_gpu_pipeline_v2.rs:487-669
over the graph kernels, src/cuda_ffi/csrc/ndt_graph_kernels.cu:47-847):
  - identical iteration count, convergence flag and status;
  - final pose within 1e-4 m and 1e-5 rad;
  - score, NVTL and transform probability within 1e-5 relative.

Newton trajectories through ill-conditioned or indefinite Hessians are chaotic: the
clamped, pseudo-inverted step amplifies a difference of one iterate, so two exact
evaluations a rounding apart reach different end points. On this workload the FP64 oracle
itself, started 1e-7 m or 1e-7 rad away, misses the bar above against its unperturbed run on
about one scan in six. A scan where the library misses the end-to-end bar must therefore
  - be one of those: the oracle from a start perturbed by 1e-7 (x, y or yaw) also misses the
    bar against itself on that scan, and
  - pass the per-iteration ("shadow") check: from every oracle iterate, one GPU iteration
    lands on the oracle's next iterate within 1e-6 m / 1e-6 rad with the score within 1e-6
    relative (1e-4 m where a point-voxel pair sits on the radius boundary: FP32 against FP64
    distance test, the correspondence counts differ).
At most MAX_CHAOTIC of the 64 scans may take that route, at most MAX_BOUNDARY iterates over
all of them the boundary bound; their ids are printed."""
import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, synth
from parity_helpers import shadow_check

pytestmark = pytest.mark.gpu

N_SCANS = 64
POS_TOL, ROT_TOL, REL_TOL = 1e-4, 1e-5, 1e-5
MAX_CHAOTIC = 12
PERTURB = 1e-7
MAX_BOUNDARY = 8


def _end_to_end_ok(got, want, compare_values=True):
    if got["iterations"] != want["iterations"] or got["converged"] != want["converged"]:
        return False
    if got["status"] != want["status"]:
        return False
    if np.abs(got["pose"][:3] - want["pose"][:3]).max() > POS_TOL:
        return False
    if np.abs(got["pose"][3:] - want["pose"][3:]).max() > ROT_TOL:
        return False
    if not compare_values:
        return True
    for k in ("score", "nvtl", "transform_probability"):
        ref = abs(want[k]) if want[k] != 0 else 1.0
        if abs(got[k] - want[k]) > REL_TOL * ref:
            return False
    return True


@pytest.fixture(scope="module")
def headline(gpu, oracle):
    import torch
    seq = synth.Sequence(seed=2, n_map=5_000_000, n_scans=1000)
    ks = list(range(2, 2 + N_SCANS))
    scans = [seq.scan(k) for k in ks]
    poses = np.stack([seq.guess(k) for k in ks])
    ctx = capi.Context()
    ctx.set_target(seq.map)
    xyz = torch.from_numpy(np.concatenate(scans).astype(np.float32)).cuda()
    offsets = np.concatenate([[0], np.cumsum([len(s) for s in scans])]).astype(np.uint64)
    tune = ctx.autotune(xyz.data_ptr(), offsets, poses, repeats=1)
    got = ctx.align_batch_device(xyz.data_ptr(), offsets, list(poses))
    grid = oracle.Grid(seq.map, 2.0)
    want = grid.align_batch(scans, poses, semantics="gpu")
    # the oracle's own sensitivity: the same scans from starts moved by PERTURB in x, y, yaw
    sensitive = set()
    for axis in (0, 1, 5):
        p2 = poses.copy()
        p2[:, axis] += PERTURB
        for i, w2 in enumerate(grid.align_batch(scans, p2, semantics="gpu")):
            if not _end_to_end_ok(w2, want[i], compare_values=False):
                sensitive.add(i)
    yield dict(seq=seq, scans=scans, poses=poses, ctx=ctx, tune=tune, got=got, want=want,
               grid=grid, sensitive=sorted(sensitive))
    ctx.close()


def _describe(got, want):
    return (f"it {got['iterations']}/{want['iterations']} "
            f"dpos {np.abs(got['pose'][:3] - want['pose'][:3]).max():.1e} "
            f"drot {np.abs(got['pose'][3:] - want['pose'][3:]).max():.1e} "
            f"dscore {abs(got['score'] - want['score']) / abs(want['score']):.1e} "
            f"dnvtl {abs(got['nvtl'] - want['nvtl']) / abs(want['nvtl']):.1e}")


def test_headline_scans_match_fp64_oracle(headline):
    h = headline
    got, want = h["got"], h["want"]
    assert len(got) == N_SCANS and all(len(s) == 20_000 for s in h["scans"])
    chaotic = [i for i in range(N_SCANS) if not _end_to_end_ok(got[i], want[i])]
    dp = [np.abs(got[i]["pose"][:3] - want[i]["pose"][:3]).max() for i in range(N_SCANS)]
    print(f"\nlaunch shape {h['tune']}; end-to-end parity on {N_SCANS - len(chaotic)}/"
          f"{N_SCANS} scans; max |dpos| over them "
          f"{max([dp[i] for i in range(N_SCANS) if i not in chaotic] or [0]):.2e} m; "
          f"scans outside the bar {chaotic}; scans where the oracle parts from itself under a "
          f"{PERTURB:g} start perturbation {h['sensitive']}")

    # shadow check of every iteration of the scans that miss the end-to-end bar, same
    # kernel form
    tune = h["tune"]
    step = capi.Context(max_iterations=1, cluster_size=tune["cluster_size"],
                        threads_per_cta=tune["threads_per_cta"],
                        max_registers=tune["registers"],
                        work_queue=tune["work_queue"] if tune["work_queue"] > 0 else -1)
    step.set_target(h["seq"].map)
    step.trace(True)
    boundary, failures = [], []
    for i in chaotic:
        fails, bnd = shadow_check(step, h["grid"], h["scans"][i], h["poses"][i])
        print(f"  scan {i}: {_describe(got[i], want[i])}; shadow: boundary iterates {bnd}, "
              f"misses {fails}")
        failures += [(i, f) for f in fails]
        boundary += [(i, k) for k in bnd]
    step.close()
    assert not failures, failures
    assert set(chaotic) <= set(h["sensitive"]), sorted(set(chaotic) - set(h["sensitive"]))
    assert len(chaotic) <= MAX_CHAOTIC, chaotic
    assert len(boundary) <= MAX_BOUNDARY, boundary


def test_headline_batch_deterministic(headline):
    """The same batch again (graph replay of the same shape): identical results bit for bit."""
    import torch
    h = headline
    xyz = torch.from_numpy(np.concatenate(h["scans"]).astype(np.float32)).cuda()
    offsets = np.concatenate([[0], np.cumsum([len(s) for s in h["scans"]])]).astype(np.uint64)
    again = h["ctx"].align_batch_device(xyz.data_ptr(), offsets, list(h["poses"]))
    for a, b in zip(h["got"], again):
        np.testing.assert_array_equal(a["pose"], b["pose"])
        assert a["score"] == b["score"] and a["nvtl"] == b["nvtl"]
        assert a["iterations"] == b["iterations"]

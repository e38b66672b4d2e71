"""Helpers shared by the GPU parity tests: the per-iteration ("shadow") check of a Newton
trajectory against the FP64 oracle's trace, and the oracle-side test for an indefinite
Hessian along a trajectory."""
import numpy as np

# per-iteration bars: the next iterate from the same start pose
STEP_POS, STEP_ROT, STEP_REL = 1e-6, 1e-6, 1e-6
# an iterate whose point-voxel pair set differs (FP32 against FP64 radius test)
BOUNDARY_POS, BOUNDARY_ROT = 1e-4, 1e-5


def shadow_check(step_ctx, grid, scan, pose, semantics="gpu"):
    """Runs one GPU iteration (step_ctx has max_iterations = 1 and tracing on) from every
    iterate of the oracle's trajectory of (scan, pose). Returns (failures, boundary):
    failures lists (iteration, dpos, drot, dscore_rel) that miss their bar; boundary lists
    the iterations whose correspondence counts differ (held to the looser bar)."""
    w, tw = grid.align_trace(scan, pose, semantics=semantics)
    starts = tw[:, 3:9]
    nexts = np.vstack([starts[1:], w["pose"][None]])
    res = step_ctx.align_multi_pose(scan, list(starts))
    failures, boundary = [], []
    for k, r in enumerate(res):
        tg = step_ctx.read_trace(k)
        same_pairs = int(tg[0, 2]) == int(tw[k, 2])
        ep = float(np.abs(r["pose"][:3] - nexts[k][:3]).max())
        er = float(np.abs(r["pose"][3:] - nexts[k][3:]).max())
        es = float(abs(tg[0, 1] - tw[k, 1]) / max(abs(tw[k, 1]), 1.0))
        if same_pairs:
            if ep > STEP_POS or er > STEP_ROT or es > STEP_REL:
                failures.append((k, ep, er, es))
        else:
            boundary.append(k)
            if ep > BOUNDARY_POS or er > BOUNDARY_ROT:
                failures.append((k, ep, er, es))
    return failures, boundary


def hessian_from_trace_row(row):
    """The 6x6 Hessian of one trace record (upper triangle at columns 15..35)."""
    H = np.zeros((6, 6))
    iu = np.triu_indices(6)
    H[iu] = row[15:36]
    return H + np.triu(H, 1).T


def trajectory_has_indefinite_hessian(grid, scan, pose, semantics="gpu"):
    """True when some iterate of the oracle's trajectory has a Hessian that is not negative
    definite: the Newton direction there comes from the eigen path, and nearby trajectories
    may separate."""
    _, tw = grid.align_trace(scan, pose, semantics=semantics)
    for row in tw:
        ev = np.linalg.eigvalsh(hessian_from_trace_row(row))
        if ev.max() >= 0.0:
            return True
    return False


def matrix_ulps(a, b):
    """Per row (one 3x3 matrix per row, 9 entries), the largest entry difference in units of
    the f32 spacing at that matrix's largest entry: the f32-ULP error of a matrix relative to
    its norm (an entry near zero gets no tighter bar than the matrix's scale)."""
    a = np.asarray(a, np.float64).reshape(len(a), -1)
    b = np.asarray(b, np.float64).reshape(len(b), -1)
    scale = np.maximum(np.abs(a).max(axis=1), np.abs(b).max(axis=1))
    spacing = np.spacing(scale.astype(np.float32)).astype(np.float64)
    spacing[spacing == 0] = np.finfo(np.float32).tiny
    return np.abs(a - b).max(axis=1) / spacing

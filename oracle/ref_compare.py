"""Prints the library's results beside the reference's own graph-path kernels and the FP64
oracle (test infrastructure; needs a GPU and the oracle/_ref cubins).

    python -m oracle.ref_compare

For each alignment: iterations (the library / FP64 oracle / reference kernels) and the largest
position difference of each pair. Where the reference departs from the FP64 evaluation of its
own algorithm, that is its FP32 error (pose state, transform, atomic sums).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from cuda_ndt_matcher_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O, ref_graph  # noqa: E402


def _dpos(a, b):
    return float(np.abs(a["pose"][:3] - b["pose"][:3]).max())


def main():
    d1, d2 = (float(np.float32(x)) for x in O.gauss_params(2.0, 0.55))
    ref = ref_graph.RefGraph()

    def map_both(ctx, pts):
        ctx.set_target(pts)
        _, means, _, icovs, _ = ctx.map_voxels()
        ref.set_map(means, icovs, 2.0)

    print("| workload | alignment | iterations ours/FP64/ref | ours-ref m | FP64-ref m | "
          "ours-FP64 m |")
    print("|---|---|---|---|---|---|")
    for seed in (1, 2, 3):
        case = synth.single_case(seed)
        g = O.Grid(case.map_points, 2.0)
        for ls in (0, 1):
            ctx = capi.Context(use_line_search=ls)
            map_both(ctx, case.map_points)
            r = ctx.align(case.scan, case.guess)
            w = ref.align(case.scan, case.guess, d1, d2, line_search=bool(ls))
            o = g.align(case.scan, case.guess, semantics="gpu", ls_candidates=8 * ls)
            print(f"| 200k-pt scene{' + line search' if ls else ''} | seed {seed} | "
                  f"{r['iterations']}/{o['iterations']}/{w['iterations']} | {_dpos(r, w):.1e} | "
                  f"{_dpos(o, w):.1e} | {_dpos(r, o):.1e} |")
    seq = synth.Sequence(seed=2, n_map=5_000_000, n_scans=24, scan_points=20_000)
    scans = [seq.scan(k) for k in range(24)]
    poses = [seq.guess(k) for k in range(24)]
    ctx = capi.Context()
    map_both(ctx, seq.map)
    got = ctx.align_batch(scans, poses)
    g = O.Grid(seq.map, 2.0)
    agree = [0, 0]
    for k in range(24):
        w = ref.align(scans[k], poses[k], d1, d2)
        o = g.align(scans[k], poses[k], semantics="gpu")
        r = got[k]
        for j, x in enumerate((r, o)):
            agree[j] += (x["iterations"] == w["iterations"] and _dpos(x, w) <= 1e-4)
        print(f"| 5M-pt map, 20k-pt scans (batch) | scan {k} | "
              f"{r['iterations']}/{o['iterations']}/{w['iterations']} | {_dpos(r, w):.1e} | "
              f"{_dpos(o, w):.1e} | {_dpos(r, o):.1e} |")
    print(f"\nsequence scans agreeing with the reference (same iterations, 1e-4 m): "
          f"ours {agree[0]}/24, FP64 oracle {agree[1]}/24")
    ref.close()


if __name__ == "__main__":
    main()

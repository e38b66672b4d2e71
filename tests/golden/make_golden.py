"""Writes reference_known_answers.json: the known-answer vectors of the reference's own
tests for the NDT hot path, transcribed from the test sources (cited per entry). The
reference is Rust and cannot be built in this environment, so these literal vectors are the
pins for the oracle (tests/test_oracle_golden.py) and, through it, for the GPU kernels."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

GOLDEN = {
    # src/ndt_cuda/src/voxel_grid/types.rs:221-235 (test_voxel_coord_from_point), res 2.0
    "voxel_coord": {
        "resolution": 2.0,
        "cases": [[[0.0, 0.0, 0.0], [0, 0, 0]],
                  [[3.5, 5.1, 1.9], [1, 2, 0]],
                  [[-3.5, -1.1, -0.1], [-2, -1, -1]]],
    },
    # src/ndt_cuda/src/voxel_grid/gpu/morton.rs:332-356 (round trip) and :358-375 (ordering)
    "morton_roundtrip": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1],
                         [100, 200, 300], [0x1FFFFF, 0x1FFFFF, 0x1FFFFF]],
    "morton_ordering": {"near": [[0, 0, 0], [1, 0, 0], [0, 1, 0]], "far": [100, 100, 100],
                        "near_max_delta": 10, "far_min_delta": 1000},
    # src/ndt_cuda/src/voxel_grid/gpu/morton.rs:377-388 (three points, res 0.5)
    "morton_codes_cpu": {"points": [[0, 0, 0], [1, 0, 0], [0, 1, 0]], "resolution": 0.5},
    # src/ndt_cuda/src/voxel_grid/gpu/radix_sort.rs:163-196 (sorted keys; equal keys keep order)
    "radix_sort": {"keys": [5, 3, 8, 1, 9, 2, 7, 4, 6, 0], "values": list(range(10)),
                   "sorted_keys": list(range(10)), "sorted_values": [9, 3, 5, 1, 7, 0, 8, 6, 2, 4],
                   "stable_keys": [1, 1, 1, 1, 1], "stable_values": [0, 1, 2, 3, 4]},
    # src/ndt_cuda/src/voxel_grid/gpu/segments.rs:170-248 and
    # src/cuda_ffi/csrc/segment_detect.cu:20-26
    "segments": [
        {"codes": [1, 1, 1, 5, 5, 9, 9, 9, 9], "ids": [0, 0, 0, 1, 1, 2, 2, 2, 2],
         "starts": [0, 3, 5], "lengths": [3, 2, 4], "num": 3},
        {"codes": [42] * 100, "starts": [0], "num": 1},
        {"codes": list(range(50)), "ids": list(range(50)), "num": 50},
        {"codes": [1, 1, 2, 2, 2, 3], "ids": [0, 0, 1, 1, 1, 2], "starts": [0, 2, 5], "num": 3},
        {"codes": [10, 10, 20, 20, 20, 30, 40, 40], "ids": [0, 0, 1, 1, 1, 2, 3, 3],
         "starts": [0, 2, 5, 6], "num": 4},
        {"codes": [], "ids": [], "starts": [], "num": 0},
    ],
    # src/ndt_cuda/src/optimization/newton.rs:206-252 (newton_step on diagonal Hessians,
    # tolerance 1e-10) and :344-403 (negative-definite tests)
    "newton": [
        {"g": [1, 2, 3, 4, 5, 6], "H_diag": [1] * 6, "delta": [-1, -2, -3, -4, -5, -6]},
        {"g": [2, 4, 6, 8, 10, 12], "H_diag": [2] * 6, "delta": [-1, -2, -3, -4, -5, -6]},
        {"g": [0] * 6, "H_diag": [1] * 6, "delta": [0] * 6},
    ],
    "newton_singular": {"g": [1, 2, 3, 4, 5, 6], "H_diag": [0] * 6},
    "negative_definite": {"min_eigenvalue": -1e-3,
                          "mixed_diag": [1.0, -1, -1, -1, -1, -1]},
    # src/ndt_cuda/src/derivatives/types.rs:201-222: d1 < 0, d2 > 0 at (2.0, 0.55);
    # (1.0, 0.3) differs from the default by more than 0.01 in d1
    "gauss": {"default": [2.0, 0.55], "custom": [1.0, 0.3], "custom_min_delta_d1": 0.01},
    # src/ndt_cuda/src/voxel_grid/types.rs:300-340 (test_regularize_covariance)
    "regularize": {"cov": [[1.0, 0, 0], [0, 1.0, 0], [0, 0, 0.0001]], "ratio": 0.01,
                   "min_ratio_after": 0.009, "identity_tol": 1e-8},
    # src/ndt_cuda/src/voxel_grid/types.rs:238-282 (test_voxel_from_statistics)
    "voxel_from_statistics": {
        "points": [[1.0, 2.0, 3.0], [1.1, 2.1, 3.1], [0.9, 1.9, 2.9], [1.05, 2.05, 3.05],
                   [0.95, 1.95, 2.95], [1.02, 2.02, 3.02], [0.98, 1.98, 2.98],
                   [1.03, 2.03, 3.03], [0.97, 1.97, 2.97], [1.0, 2.0, 3.0]],
        "mean": [1.0, 2.0, 3.0], "mean_tol": 0.1, "cov_norm_max": 0.1, "identity_tol": 0.01},
    # src/ndt_cuda/src/derivatives/cpu.rs:567-660 (transform_point cases)
    "transform_point": [
        {"point": [1, 2, 3], "pose": [0, 0, 0, 0, 0, 0], "out": [1, 2, 3]},
        {"point": [1, 2, 3], "pose": [1, 2, 3, 0, 0, 0], "out": [2, 4, 6]},
        {"point": [1, 0, 0], "pose": [0, 0, 0, 0, 0, 1.5707963267948966], "out": [0, 1, 0]},
    ],
    # src/ndt_cuda/src/derivatives/cpu.rs:695-715: score at the mean equals -d1
    "score_at_mean": {"resolution": 2.0, "outlier": 0.55},
    # src/ndt_cuda/src/test_utils.rs:19-61: half-cube map (3 planes, 20 m, 0.2 m spacing)
    "half_cube": {"length": 20.0, "interval": 0.2, "num_points": 30603},
}

if __name__ == "__main__":
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(GOLDEN, f, indent=1)
    print("wrote reference_known_answers.json")

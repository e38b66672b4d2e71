"""The C-ABI library builds, loads and exports every symbol include/ndt_gb300.h declares;
host-side logic that needs no GPU. No compute calls are made here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from cuda_ndt_matcher_gb300 import capi, matcher
from tests.conftest import has_gpu

HDR = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "ndt_gb300.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.findall(r"^\s*(?:int|void\*|const char\*)\s+(ndt_\w+)\s*\(", src, flags=re.M)


def test_header_and_binding_agree():
    decl = declared_functions()
    assert len(decl) >= 20
    assert sorted(decl) == sorted(capi.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = capi.load()
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing
    out = os.popen(f"nm -D --defined-only {capi.lib_path()}").read()
    for f in declared_functions():
        assert re.search(rf"\bT {f}\b", out), f


def test_struct_layouts():
    assert C.sizeof(capi.Result) == 6 * 8 + 3 * 8 + 36 * 8 + 6 * 4
    assert C.sizeof(capi.Config) == 96
    assert C.sizeof(capi.TuneResult) == 48
    assert C.sizeof(capi.PNetConfig) == 48
    assert C.sizeof(capi.Scan) == 8 + 8 + 48
    assert C.sizeof(capi.ParticleConfig) == 4 + 4 + 4 * 8 + 8
    assert C.sizeof(capi.PoseEstimate) == 12 * 8 + 3 * 8 + 4 * 4
    assert C.sizeof(capi.Stats) == 19 * 8
    assert C.sizeof(capi.MapInfo) == 4 * 8 + 4 + 3 * 12 + 2 * 4 + 2 * 4
    assert C.sizeof(capi.PNetStats) == 5 * 8


def test_config_defaults_mirror_reference():
    """NdtScanMatcherConfig::default (src/ndt_cuda/src/ndt.rs:90-107) and the graph kernel's
    neighbour cap (src/cuda_ffi/csrc/ndt_graph_common.cuh:21)."""
    cfg = capi.default_config()
    assert cfg.resolution == 2.0 and cfg.max_iterations == 30
    assert cfg.trans_epsilon == 0.01 and cfg.step_size == 0.1 and cfg.outlier_ratio == 0.55
    assert cfg.min_points_per_voxel == 6 and abs(cfg.eigenvalue_ratio - 0.01) < 1e-9
    assert cfg.max_neighbors == 8 and cfg.min_correspondences == 10
    assert cfg.hash_capacity_factor == 2
    assert cfg.use_line_search == 0  # NdtScanMatcherConfig::default, ndt.rs:99


def test_line_search_config_checked():
    """The configuration is checked before any device call: use_line_search is 0 or 1 (both
    semantics take it: the graph path's candidates, the CPU path's More-Thuente search)."""
    with pytest.raises(capi.NdtError) as e:
        capi.Context(use_line_search=2)
    assert e.value.code == -1


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_context_fails_loudly_without_device():
    with pytest.raises(capi.NdtError) as e:
        capi.Context()
    assert e.value.code == -9


def test_pose_isometry_round_trip():
    rng = np.random.default_rng(0)
    for _ in range(50):
        p = np.concatenate([rng.uniform(-100, 100, 3), rng.uniform(-1.2, 1.2, 3)])
        T = matcher.pose_vector_to_isometry(p)
        assert np.allclose(T[:3, :3] @ T[:3, :3].T, np.eye(3), atol=1e-12)
        q = matcher.isometry_to_pose_vector(T)
        assert np.allclose(q, p, atol=1e-9)


def test_isometry_matches_oracle_zyx(oracle):
    p = np.array([1.0, 2.0, 3.0, 0.1, -0.2, 0.3])
    assert np.allclose(matcher.pose_vector_to_isometry(p)[:3], oracle.pose_T34_zyx(p))


def test_builder_mirrors_reference_names():
    b = matcher.NdtScanMatcher.builder().resolution(1.0).max_iterations(10) \
        .transformation_epsilon(0.02).step_size(0.2).outlier_ratio(0.5).use_gpu(True)
    c = b.config
    assert (c.resolution, c.max_iterations, c.trans_epsilon, c.step_size, c.outlier_ratio,
            c.use_gpu) == (1.0, 10, 0.02, 0.2, 0.5, True)


def test_reference_kernel_driver_builds():
    """The host driver of the reference's own graph-path kernels builds and exports its entry
    points, and the cubins it loads are present (nothing runs without a GPU)."""
    import shutil
    import subprocess
    from oracle import build as ob, ref_graph
    lib = ob.build_ref_driver()
    if shutil.which("nm") is None:
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True,
                         text=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert {"rg_open", "rg_set_map", "rg_align", "rg_eval", "rg_query", "rg_close",
            "rg_error"} <= names
    if not ob.build_ref_cubins():  # compiled where the reference sources are
        pytest.skip("neither the reference sources nor prebuilt cubins are here")
    assert ref_graph.available()


def test_tpe_proposals_match_oracle(oracle):
    """The guided particles' TPE proposals (ndt_tpe_propose, host code of the library) equal
    the oracle's restatement bit for bit: random trial sets, ties in the scores, the good set
    at its bounds (1 and 10), yaw differences across the wrap."""
    rng = np.random.default_rng(7)
    prior = np.array([10.0, -5.0, 0.3, 0.0, 0.0, 3.0])
    for n in (1, 5, 12, 57, 150, 199):
        t = np.column_stack([prior[0] + rng.normal(0, 1.5, n), prior[1] + rng.normal(0, 1.5, n),
                             rng.uniform(-np.pi, np.pi, n), np.exp(-rng.uniform(0, 30, n) / 10)])
        t[::7, 3] = t[0, 3]  # equal scores keep their arrival order
        for k in (100, 137):
            got = capi.tpe_propose(3, k, prior, t, seed=11, xy_range=2.0)
            want = oracle.tpe_propose(prior, 3, k, t, seed=11, xy_range=2.0)
            np.testing.assert_array_equal(got, want)
    # no trials: the particle's own draw
    np.testing.assert_array_equal(capi.tpe_propose(0, 5, prior, np.zeros((0, 4))),
                                  oracle.particle(prior, 0, 5))

"""GB300-native (sm_103a) NDT scan matching: a drop-in for cuda_ndt_matcher's hot path.

The compute runs in libndt_gb300.so (hand-written CUDA behind a C ABI, include/ndt_gb300.h);
this package holds the host-side mirror of the reference's NdtScanMatcher API, the ctypes
binding and the seeded synthetic workload generator.
"""
from .capi import Context, NdtError, load as load_library  # noqa: F401
from .matcher import (AlignResult, NdtScanMatcher, NdtScanMatcherBuilder,  # noqa: F401
                      NdtScanMatcherConfig, isometry_to_pose_vector, pose_vector_to_isometry,
                      translation)

__all__ = ["Context", "NdtError", "load_library", "AlignResult", "NdtScanMatcher",
           "NdtScanMatcherBuilder", "NdtScanMatcherConfig", "isometry_to_pose_vector",
           "pose_vector_to_isometry", "translation"]

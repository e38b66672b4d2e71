"""Build recipe for the package's native libraries (no cmake, no pip).

- libndt_gb300.so : the sm_103a CUDA kernels + C-ABI (nvcc, one -gencode, -lineinfo)
- libndt_synth.so : seeded procedural maps / lidar scans for tests and benchmarks (gcc)

Translation units compile in parallel; outputs land in cuda_ndt_matcher_gb300/_build/.
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
CUDA_LIB = os.path.join(OUT, "libndt_gb300.so")
SYNTH_LIB = os.path.join(OUT, "libndt_synth.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["voxel_build.cu", "ndt_align.cu", "ndt_score.cu", "ndt_api.cu", "tc_gemm.cu",
              "mlp.cu"]
CU_DEPS = ["ndt_common.cuh", "ndt_internal.h"]


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_synth(force=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "synth.c")
    if force or _newer(SYNTH_LIB, [src]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-o", SYNTH_LIB + ".tmp", src, "-lm"])
        os.replace(SYNTH_LIB + ".tmp", SYNTH_LIB)
    return SYNTH_LIB


def build_cuda(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdr = os.path.join(INCLUDE, "ndt_gb300.h")
    deps_common = [os.path.join(CSRC, d) for d in CU_DEPS] + [hdr]
    objs = []
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _newer(obj, [src] + deps_common):
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(CUDA_LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", CUDA_LIB + ".tmp"] + objs +
             ["-lcudart"])
        os.replace(CUDA_LIB + ".tmp", CUDA_LIB)
    if verbose:
        return "\n".join(logs)
    return CUDA_LIB


def build_all(force=False):
    return build_synth(force), build_cuda(force)


if __name__ == "__main__":
    import sys
    print(build_synth(True))
    print(build_cuda(True, verbose="-v" in sys.argv))

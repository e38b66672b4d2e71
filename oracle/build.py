"""Build recipe for the oracle library (gcc, no external dependencies).

Output: oracle/_build/libndt_oracle.so. -ffp-contract=off makes every floating-point
operation a single IEEE rounding on both x86-64 and aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libndt_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ndt_oracle.c")
    hdr = os.path.join(HERE, "ndt_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB + ".tmp", src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: NDT_REFERENCE_DIR, else the container's read-only mount; the GPU
# machine has neither and uses the cubins built here
REF_ROOT = os.environ.get("NDT_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src", "cuda_ffi", "csrc")
# the reference's graph-path kernels and voxel hash, compiled unmodified into device-only
# cubins with the reference's own flags (-O3, one architecture; src/cuda_ffi/build.rs:131-148)
REF_CUBINS = {"ndt_graph_kernels.cubin": "ndt_graph_kernels.cu",
              "voxel_hash.cubin": "voxel_hash.cu"}
REF_DRIVER = os.path.join(OUT_DIR, "libref_graph.so")


def build_ref_cubins(force: bool = False) -> bool:
    """Compiles the reference's CUDA sources where they lie into oracle/_ref (only where the
    reference is present; the cubins hold no host code, so they run on any host)."""
    if not os.path.isdir(REF_SRC):
        return all(os.path.exists(os.path.join(REF_DIR, c)) for c in REF_CUBINS)
    os.makedirs(REF_DIR, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    for cubin, src in REF_CUBINS.items():
        out, path = os.path.join(REF_DIR, cubin), os.path.join(REF_SRC, src)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(path):
            continue
        subprocess.check_call([nvcc, "-cubin", "-O3", "-arch=sm_103a", "-I", REF_SRC,
                               "-o", out + ".tmp", path])
        os.replace(out + ".tmp", out)
    return True


def _cuda_stub_dir():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cands = [os.path.join(home, "lib64", "stubs")]
    tdir = os.path.join(home, "targets")
    if os.path.isdir(tdir):
        cands += [os.path.join(tdir, t, "lib", "stubs") for t in sorted(os.listdir(tdir))]
    for c in cands:
        if os.path.exists(os.path.join(c, "libcuda.so")):
            return home, c
    raise RuntimeError("libcuda.so stub not found under " + home)


def build_ref_driver(force: bool = False) -> str:
    """The host side that runs the reference cubins (oracle/ref_graph.c, CUDA driver API)."""
    src = os.path.join(HERE, "ref_graph.c")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(REF_DRIVER)
            and os.path.getmtime(REF_DRIVER) >= os.path.getmtime(src)):
        return REF_DRIVER
    home, stubs = _cuda_stub_dir()
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared",
                           "-I", os.path.join(home, "include"), "-o", REF_DRIVER + ".tmp", src,
                           "-L", stubs, "-lcuda"])
    os.replace(REF_DRIVER + ".tmp", REF_DRIVER)
    return REF_DRIVER


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref_cubins(force=True), build_ref_driver(force=True))

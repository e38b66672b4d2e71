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


if __name__ == "__main__":
    print(build(force=True))

"""Build recipe for the CPU oracle (test infrastructure, never the product).

Compiles oracle/letkf_oracle.c into oracle/_build/liboracle.so with gcc.
-ffp-contract=off keeps every multiply and add separately rounded, as the
reference's gfortran -O2 x86-64 build does.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "letkf_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "letkf_gpu.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-std=gnu11", "-Wall", "-Wno-unused-function",
           "-o", LIB + ".tmp", SRC, "-ldl", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

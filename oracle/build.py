"""Build recipe for the FP64 C oracle (test infrastructure only).

Compiles oracle/mgbf_oracle.c into oracle/_build/libmgbf_oracle.so with gcc
and OpenMP.  Only the test suite, the smoke check and the benchmark's CPU
baseline load the result; the shipped library never does.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmgbf_oracle.so")
SRC = [os.path.join(HERE, "mgbf_oracle.c")]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SRC + [os.path.join(HERE, "mgbf_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
           "-ffp-contract=off", "-o", tmp] + SRC + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

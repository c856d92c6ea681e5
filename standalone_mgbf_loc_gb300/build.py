"""Build libmgbf.so (sm_103a CUDA kernels + C++ host orchestration) in-tree.

Each translation unit is compiled in parallel with nvcc for
`-gencode arch=compute_103a,code=sm_103a`; the result lands in
standalone_mgbf_loc_gb300/_lib/libmgbf.so.  No torch dependency: the library
is a plain C-ABI shared object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIB_DIR, "libmgbf.so")
OBJ_DIR = os.path.join(ROOT, "_build", "obj")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = [
    "mgbf_capi.cpp",
    "mgbf_setup.cpp",
    "mgbf_kernels.cu",
    "mgbf_hbeta_f32.cu",
    "mgbf_hbeta_f32_b.cu",
    "mgbf_hbeta_f64.cu",
    "mgbf_hbeta_bf16.cu",
    "mgbf_hbeta_bf16_b.cu",
    "mgbf_noalloc.cu",
    "mgbf_xfer.cu",
    "mgbf_rad3.cu",
    "mgbf_dibeta.cu",
    "mgbf_lin3.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmgbf")
    return cand


def _deps() -> list:
    out = [os.path.join(INCLUDE, "mgbf.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _compile(src: str) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ_DIR, src + ".o")
    cmd = [_nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd += ARCH + ["-Xptxas", "-O3"]
    else:
        cmd += ["-x", "cu"] + ARCH
    cmd += ["-c", path, "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    newest = max(os.path.getmtime(d) for d in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run([_nvcc(), "-shared", "-o", tmp] + ARCH + objs + ["-cudart=static"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv))

"""In-tree build of libgkrt.so for sm_103a.

Each .cu translation unit is compiled in parallel with nvcc (one -gencode, sm_103a) and
linked into gknextengine_gb300/_lib/libgkrt.so, which the ctypes binding loads. Kernels
are compiled with -fmad=false and host code with -ffp-contract=off: fused multiply-adds
appear only where the source writes them, so float results do not depend on compiler
contraction choices (the host-built emitter table must match the oracle's bit for bit).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libgkrt.so")
# The checked build (GKRT_CHECKED): traversal tests every node, triangle and instance index
# against its array before the access and records kErrBounds instead of reading out of range;
# the sanitizer-style variant of the library for tests (environment GKRT_LIBRARY selects it).
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libgkrt_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-Xptxas", "-v"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgkrt")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(HERE, "..", "include", "gkrt.h"))
    return hdrs


def _compile(src: str, log_dir: str, extra=()) -> str:
    obj = os.path.join(log_dir, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(os.path.join(log_dir, os.path.basename(src) + ".ptxas.txt"), "w") as f:
        f.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-4000:]}")
    return obj


def build(force: bool = False, jobs: int | None = None, checked: bool = False) -> str:
    srcs = sources()
    lib = CHECKED_LIB_PATH if checked else LIB_PATH
    obj_dir = os.path.join(BUILD_DIR, "checked") if checked else BUILD_DIR
    newest = max(os.path.getmtime(p) for p in srcs + _deps() + [__file__])
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= newest:
        return lib
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    extra = ["-DGKRT_CHECKED"] if checked else []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, obj_dir, extra), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs + ["-ldl"]   # NVTX loads tools
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True))

"""Builds libqobgpu.so (the C-ABI library of hand-written sm_103a kernels).

Each translation unit is compiled by nvcc in parallel, then linked into
qobgpu/libqobgpu.so.  Only one target is built: -gencode
arch=compute_103a,code=sm_103a.  No cmake; runs the same on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "qobgpu", "libqobgpu.so")
# the bounds-checked build (-DQOB_DEBUG_BOUNDS): gathered indices checked on the
# device and reported through qob_device_status; built on request for its tests
DEBUG_OUT_DIR = os.path.join(HERE, "_build_debug")
DEBUG_LIB = os.path.join(HERE, "qobgpu", "libqobgpu_debug.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall", "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=(), debug_bounds: bool = False) -> str:
    lib_path = DEBUG_LIB if debug_bounds else LIB
    out_dir = DEBUG_OUT_DIR if debug_bounds else OUT_DIR
    if debug_bounds:
        extra = list(extra) + ["-DQOB_DEBUG_BOUNDS"]
    if not force and not _stale(lib_path):
        return lib_path
    os.makedirs(out_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(out_dir, src[:-3] + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = lib_path + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else [],
                debug_bounds="--debug-bounds" in sys.argv))

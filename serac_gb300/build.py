"""Builds the sfx CUDA library in-tree for sm_103a.

Every ``serac_gb300/csrc/*.cu`` file is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``serac_gb300/libsfx_gb300.so``.  Objects go to ``serac_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libsfx_gb300.so")
BUILD = os.path.join(HERE, "_build")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "--extended-lambda",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))


def _headers_mtime():
    files = glob.glob(os.path.join(ROOT, "include", "**", "*"), recursive=True)
    files += glob.glob(os.path.join(HERE, "csrc", "*.hpp"))
    return max((os.path.getmtime(f) for f in files if os.path.isfile(f)), default=0.0)


def _compile(src, verbose=False, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _headers_mtime()):
        return obj, ""
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "csrc"),
           "-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{p.stderr[-8000:]}")
    return obj, p.stderr


def build(verbose=False, jobs=None, extra=()):
    """Compile and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, extra), srcs))
    objs = [r[0] for r in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", LIB, *objs, "-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stderr[-8000:]}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

"""Builds libsledgehamr_gb300.so (the CUDA library behind
include/sledgehamr_gb300.h) in-tree, for sm_103a only.

Every translation unit under csrc/ is compiled by nvcc in parallel and the
objects are linked into sledgehamr_gb300/libsledgehamr_gb300.so.  Objects go
to sledgehamr_gb300/_build/.  A unit is recompiled when it or any header of
the package or of include/ is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsledgehamr_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-fopenmp",
    "-I" + os.path.join(ROOT, "include"),
    "-I" + os.path.join(ROOT, "include", "sledgehamr"),
    "-diag-suppress", "177,550,20012",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build")
    return cand


def _headers() -> list[str]:
    pats = [os.path.join(PKG, "csrc", "*.h"), os.path.join(PKG, "csrc", "*.cuh"),
            os.path.join(PKG, "projects", "*", "*.h"),
            os.path.join(ROOT, "include", "*.h"), os.path.join(ROOT, "include", "sledgehamr", "*.h")]
    out = []
    for p in pats:
        out += glob.glob(p)
    return out


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return m < os.path.getmtime(src) or m < hdr_mtime


def build(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(PKG, "csrc", "*.cu")))
    hdr_mtime = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    todo = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, s, hdr_mtime):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(f"compiled {os.path.basename(s)}", file=sys.stderr)
        return o

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(compile_one, todo))
    if todo or not os.path.exists(LIB):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcufft", "-lcudart",
                                                               "-Xcompiler", "-fopenmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))

"""Build recipe of the CUDA engine: nvcc for sm_103a, in-tree output.

``python -m q6_gb300.build`` (or ``__graft_entry__.build()``) compiles the
translation units of ``q6_gb300/csrc`` in parallel and links
``q6_gb300/_build/libqnb.so``.  Only the sm_103a (GB300) target is built.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libqnb.so")
SOURCES = ["qnb_kernels.cu", "qnb_host.cpp", "qnb_noalloc.cu", "qmd_kernels.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-diag-suppress", "177"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src, os.path.join(SRC, "qnb_internal.h"),
            os.path.join(HERE, "..", "include", "qnb.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    objs, jobs = [], []
    for s in SOURCES:
        src = os.path.join(SRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj]
            if s.endswith(".cpp"):
                cmd = [nvcc(), *FLAGS, "-x", "c++", "-c", src, "-o", obj]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for cmd, r in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}")
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

"""Build libsfmm_gb300.so in-tree: nvcc for sm_103a, one object per source,
compiled in parallel, then linked with the static CUDA runtime.

    python -m solidfmm_gb300.build [--clean]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CXX = os.path.join(PKG, "cxx")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsfmm_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]


def _sources():
    out = []
    for d in (CSRC, CXX):
        if not os.path.isdir(d):
            continue
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def _headers():
    hs = []
    for d in (CSRC, CXX, INCLUDE, os.path.join(INCLUDE, "solidfmm")):
        if os.path.isdir(d):
            hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".hpp", ".cuh"))]
    return hs


def _obj(src):
    base = os.path.relpath(src, PKG).replace(os.sep, "_")
    return os.path.join(BUILD, base + ".o")


def _compile(src):
    obj = _obj(src)
    cmd = [NVCC] + COMMON + ARCH + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    hdr_mtime = max((os.path.getmtime(h) for h in _headers()), default=0)
    todo = []
    for s in srcs:
        o = _obj(s)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_mtime):
            todo.append(s)
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4, 16)
    if todo:
        with cf.ThreadPoolExecutor(jobs) as ex:
            list(ex.map(_compile, todo))
    objs = [_obj(s) for s in srcs]
    if force or todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIBDIR, ignore_errors=True)


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(force="--force" in sys.argv))

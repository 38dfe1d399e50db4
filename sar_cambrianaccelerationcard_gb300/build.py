"""Builds libsarbp.so in-tree from csrc/ with nvcc for sm_103a.

One translation unit per nvcc process, compiled in parallel, then linked as a
shared library with the static CUDA runtime.  No cmake.
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
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsarbp.so")
SOURCES = ["rc.cu", "bp.cu", "synth.cu", "probe.cu", "noalloc.cu", "autofocus.cu", "wk.cu", "ceos.cu", "plan.cpp", "serve.cpp", "api.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]


def _compile(src: str, extra=(), build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".h")] + \
        [os.path.join(ROOT, "include", "sarbp.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *_flags(extra), "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu", *_flags(extra), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, extra=(), lib: str = LIB, build_dir: str = BUILD) -> str:
    """Compile (incrementally) and link.  `extra` adds nvcc flags (e.g. -D
    tuning macros); `lib`/`build_dir` place a variant build elsewhere."""
    os.makedirs(build_dir, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, build_dir), SOURCES))
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(o) for o in objs):
        return lib
    cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-cudart", "static", "-Xlinker", "--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)

"""In-tree build of ``libfame_gb300.so`` for sm_103a.

Every CUDA translation unit is compiled by nvcc in parallel
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``), host C++ by g++,
and the objects are linked into ``fame/libfame_gb300.so``.  Objects go to
``_build/`` beside the package (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout[-4000:])
    return r.stdout


def sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    return cu, cpp


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(os.path.dirname(ROOT), "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile and link; returns the library path.  Incremental on mtimes."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = sources()
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    cmds = []
    objs = []
    for s in cu:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, s):
            cmds.append([nvcc] + NVFLAGS + ["-c", s, "-o", o])
    for s in cpp:
        o = os.path.join(BUILD, os.path.basename(s)[:-4] + ".o")
        objs.append(o)
        if _stale(o, s):
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(jobs) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out:
                print(out)
    lib = os.path.join(PKG, "libfame_gb300.so")
    tmp = lib + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, lib)
    return lib

"""Build libpbd_gb300.so from csrc/*.cu with nvcc for sm_103a.

    python -m positionbaseddynamicsold_gb300.build

The solver and collision translation units are compiled with -fmad=false:
their arithmetic mirrors the reference's, where every product is rounded
before the following add.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpbd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "pbd_sort.cu": [],
    "pbd_object.cu": ["-fmad=false"],
    "pbd_collision.cu": ["-fmad=false"],
    "pbd_mesh.cu": ["-fmad=false"],
    "pbd_edge.cu": ["-fmad=false"],
    "pbd_noalloc.cu": [],
    "pbd_mlp.cu": [],
    "pbd_solve.cu": [],
    "pbd_io.cpp": [],
}
HEADERS = ["pbd_common.cuh", "pbd_project.cuh", "pbd_ccd.cuh"]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout[-6000:]))
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    common = [nvcc, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC"] + ARCH + inc
    if verbose:
        common += ["-Xptxas", "-v"]
    hdr_t = max(os.path.getmtime(os.path.join(CSRC, h)) for h in HEADERS)
    hdr_t = max(hdr_t, os.path.getmtime(os.path.join(ROOT, "include", "pbd_c.h")))
    jobs, objs = [], []
    for src, extra in SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            jobs.append(common + extra + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

"""Build recipe for the oracle (test infrastructure, never the product).

* ``build_oracle()`` compiles the C restatement ``oracle/pbd_oracle.c`` into
  ``oracle/_build/liboracle.so`` (gcc, ``-ffp-contract=off`` so float
  expressions round like the reference's x86-64 host code on every host).
* ``build_ref(ref_root)`` compiles the reference's own CPU path from its
  sources where they lie (``ref_root`` = the reference checkout) together with
  ``oracle/ref_adapter.cpp`` into ``oracle/_ref/libpbdref.so``.  It is used
  only to pin the oracle and to regenerate ``tests/golden``; the reference
  checkout exists only on the development machine.

Run ``python oracle/build_oracle.py [--ref /path/to/reference]``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_SUBDIR = os.path.join("PositionBasedDynamicsCUDA", "PositionBasedDynamicsCUDA")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(REF_OUT, "libpbdref.so")


def _run(cmd):
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), res.stdout[-4000:]))
    return res.stdout


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "pbd_oracle.c"), os.path.join(HERE, "pbd_oracle.h")]
    if force or _stale(ORACLE_SO, srcs):
        cc = os.environ.get("CC", "gcc")
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        base = [cc, "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-ffp-contract=off", "-fPIC",
                "-shared", "-o", tmp, srcs[0], "-lm"]
        # OpenMP spreads the independent loops over host threads when the
        # compiler has it; without it the same code runs on one thread
        try:
            _run(base + ["-fopenmp"])
        except RuntimeError:
            _run(base)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def find_reference(ref_root: str | None = None) -> str | None:
    """The reference's source folder: the argument, else PBD_REFERENCE_ROOT,
    else the read-only checkout's mount point on the development machine
    (this recipe is the one place that reads the sources there; the GPU
    host has no checkout and uses the oracle alone)."""
    cands = [ref_root, os.environ.get("PBD_REFERENCE_ROOT"), "/root/reference"]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, REF_SUBDIR)):
            return os.path.join(c, REF_SUBDIR)
    return None


def _function_text(path: str, signature: str) -> str:
    """The source text of one function of a reference file: from the line
    holding `signature` to its closing brace (braces counted)."""
    with open(path, encoding="utf-8-sig", errors="replace") as f:
        text = f.read()
    i = text.index(signature)
    i = text.rfind("\n", 0, i) + 1
    j = text.index("{", i)
    depth = 0
    for k in range(j, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[i:k + 1]
    raise ValueError("unbalanced braces after " + signature)


def _kernel_host_unit(src: str) -> str:
    """oracle/_ref/ref_kernel_host.cpp: ProjectContraintsGPUKernel and the
    Distance it calls (P/PBD_cuda.cu), compiled for the host as written,
    with threadIdx / blockIdx / blockDim as host variables; the entry
    ref_project_colored_gpu_kernel runs one launch per color workset, every
    index of it (the intended launch, without the integer-division grid)."""
    pbd = os.path.join(src, "PBD_cuda.cu")
    dist = _function_text(pbd, "KERNEL_FUNC float Distance(float3 p1, float3 p2)")
    kern = _function_text(pbd, "void __global__ ProjectContraintsGPUKernel(")
    return "\n".join([
        "// generated by oracle/build_oracle.py from the reference's PBD_cuda.cu",
        '#include "PBD_Basic.cuh"',
        "static uint3 refk_tid, refk_bid;",
        "static dim3 refk_bdim;",
        "#define threadIdx refk_tid",
        "#define blockIdx refk_bid",
        "#define blockDim refk_bdim",
        "#define Distance refk_Distance",
        "#define ProjectContraintsGPUKernel refk_ProjectContraintsGPUKernel",
        "static " + dist,
        "static " + kern,
        'extern "C" void ref_project_colored_gpu_kernel(',
        "    int resY, int n_worksets, const int *worksets, int it0, int it1,",
        "    int *sortedPrimId, int *indices, int *constraintType, float *massBuffer,",
        "    float *restLengthBuffer, float *stiffnessBuffer, int2 *primList,",
        "    float3 *prdPBuffer, float3 *restBuffer) {",
        "    for (int it = it0; it < it1; ++it)",
        "        for (int w = 0; w < n_worksets; ++w) {",
        "            int start = worksets[2 * w], num = worksets[2 * w + 1];",
        "            refk_bdim = dim3(512, 1, 1);",
        "            for (int idx = 0; idx < num; ++idx) {",
        "                refk_bid = make_uint3(idx / 512, 0, 0);",
        "                refk_tid = make_uint3(idx % 512, 0, 0);",
        "                refk_ProjectContraintsGPUKernel(resY, start, num, it, sortedPrimId,",
        "                    indices, constraintType, massBuffer, restLengthBuffer,",
        "                    stiffnessBuffer, primList, prdPBuffer, restBuffer);",
        "            }",
        "        }",
        "}",
        ""])


def build_ref(ref_root: str | None = None, force: bool = False) -> str | None:
    """Compile the reference CPU path; returns the .so path or None if the
    reference sources are not present on this machine."""
    src = find_reference(ref_root)
    if src is None or shutil.which("nvcc") is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc")))
    incs = ["-I" + src, "-I" + os.path.join(cuda, "include"),
            "-I" + os.path.join(cuda, "include", "cccl")]
    adapter = os.path.join(HERE, "ref_adapter.cpp")
    units = [
        ("PBD_cuda.cu", ["nvcc", "-std=c++17", "-O2", "-Xcompiler",
                         "-fPIC,-fpermissive,-ffp-contract=off", "-w"]),
        ("CCD.cpp", None), ("SpatialHashSystem.cpp", None), ("timer.cpp", None),
    ]
    gxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-fpermissive", "-ffp-contract=off", "-w",
           "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP"]
    jobs = []
    objs = []
    for name, cmd in units:
        s = os.path.join(src, name)
        o = os.path.join(REF_OUT, name + ".o")
        objs.append(o)
        if force or _stale(o, [s]):
            jobs.append((cmd or gxx) + incs + ["-c", s, "-o", o])
    ao = os.path.join(REF_OUT, "ref_adapter.o")
    objs.append(ao)
    if force or _stale(ao, [adapter]):
        jobs.append(gxx + incs + ["-c", adapter, "-o", ao])
    # the GPU projection kernel's own code, compiled for the host
    kcpp = os.path.join(REF_OUT, "ref_kernel_host.cpp")
    ko = os.path.join(REF_OUT, "ref_kernel_host.o")
    objs.append(ko)
    pbd_src = os.path.join(src, "PBD_cuda.cu")
    if force or _stale(ko, [pbd_src, os.path.abspath(__file__)]):
        with open(kcpp, "w") as f:
            f.write(_kernel_host_unit(src))
        jobs.append(gxx + incs + ["-c", kcpp, "-o", ko])
    with ThreadPoolExecutor(max_workers=5) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not os.path.exists(REF_SO):
        _run(["nvcc", "-shared", "-o", REF_SO] + objs + ["-lcudart"])
    return REF_SO


if __name__ == "__main__":
    ref = None
    if "--ref" in sys.argv:
        ref = sys.argv[sys.argv.index("--ref") + 1]
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(ref, force="--force" in sys.argv))

"""Builds lagrbf_gb300/liblagrbf.so (CUDA kernels for sm_103a + the C host layer) in-tree.

The CUDA translation units compile in parallel; the result is a self-contained shared library
(static cudart) exporting the C-ABI declared in include/lagrbf.h.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblagrbf.so")

CU_SOURCES = ["lgb_bin.cu", "lgb_eval32_3d.cu", "lgb_eval32_2d.cu", "lgb_eval64.cu", "lgb_factor.cu", "lgb_step.cu",
              "lgb_noalloc.cu"]
C_SOURCES = ["lgb_host.c", "lgb_io.c", "lgb_serve.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc flags for tuning builds, e.g. LAGRBF_NVCC_FLAGS="-DLGB_X2_UNROLL=2" (default: none)
EXTRA = os.environ.get("LAGRBF_NVCC_FLAGS", "").split()


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "lagrbf.h"))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", *EXTRA,
                         "-Xptxas", "-v" if verbose else "-O3", "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc", "-std=gnu11", "-O3", "-g", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter",
                         "-ffp-contract=off", "-fvisibility=hidden", "-I" + os.path.join(cuda, "include"),
                         "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", *ARCH, "-cudart", "static", "-o", LIB, *objs, "-lpthread", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

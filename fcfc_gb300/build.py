"""Build libfcfcg.so in-tree: CUDA kernels for sm_103a (nvcc) and the C host
layer (gcc), linked with the static CUDA runtime.

    python -m fcfc_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libfcfcg.so")

CU_SOURCES = ["prep.cu", "count.cu", "count32_box.cu", "count32_survey.cu",
              "count32_batch.cu", "count32_adj.cu", "cnvt.cu", "probe.cu"]
C_SOURCES = ["bins.c", "ctx.c", "epilogue.c", "cnvt.c"]
HEADERS = ["fcfcg_internal.h", "legauss_tab.h", "count_common.cuh", "count32.cuh",
           os.path.join("..", "..", "include", "fcfcg.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode:
        raise RuntimeError("build failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + C_SOURCES]
    drv = [os.path.join(CSRC, "driver", s) for s in DRIVER_SOURCES] + \
        [os.path.join(CSRC, "driver", h) for h in ("catalog.h", "expr.h")]
    bins = [os.path.join(BINDIR, n) for n in DRIVERS]
    if not force and _newer(LIB, srcs + hdrs + [__file__]) and \
            all(_newer(b, drv + [LIB]) for b in bins):
        return LIB
    jobs = []
    for s in CU_SOURCES:
        o = os.path.join(OBJDIR, s + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                     "-I", CSRC, "-c", os.path.join(CSRC, s), "-o", o])
    for s in C_SOURCES:
        o = os.path.join(OBJDIR, s + ".o")
        jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off",
                     "-fno-fast-math", "-Wall", "-Wextra", "-Wno-unused-parameter",
                     "-I", os.path.join(cuda, "include"), "-I", CSRC,
                     "-c", os.path.join(CSRC, s), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(OBJDIR, s + ".o") for s in CU_SOURCES + C_SOURCES]
    tmp = LIB + ".tmp%d" % os.getpid()
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lm"])
    os.replace(tmp, LIB)
    build_drivers()
    return LIB


DRIVER_SOURCES = ["main.c", "conf.c", "catalog.c", "expr.c"]
DRIVERS = {"FCFC_2PT_BOX_GPU": [], "FCFC_2PT_GPU": ["-DFCFCG_SURVEY"]}
BINDIR = os.path.join(HERE, "bin")


def build_drivers():
    """The command line drivers (C, linked against libfcfcg.so)."""
    os.makedirs(BINDIR, exist_ok=True)
    src = [os.path.join(CSRC, "driver", s) for s in DRIVER_SOURCES]
    jobs = []
    for name, defs in DRIVERS.items():
        out = os.path.join(BINDIR, name)
        jobs.append(["gcc", "-O2", "-std=c11", "-ffp-contract=off",
                     "-fno-fast-math", "-Wall", *defs, "-o", out, *src,
                     "-L", LIBDIR, "-lfcfcg", "-Wl,-rpath,$ORIGIN/../lib",
                     "-lm", "-lpthread"])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)

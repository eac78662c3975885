"""Build libcfgb.so in-tree: the sm_103a kernels and the C ABI.

Kernels are compiled by nvcc for sm_103a only; the host translation units by g++ with
-ffp-contract=off (the mesh geometry must round like a plain FP64 evaluation of the
reference formulas).  The units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcfgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"

CU_SOURCES = ["cf_kernels.cu", "cf_edges_1.cu", "cf_edges_2.cu", "cf_edges_3.cu", "cf_edges_4.cu", "cf_noalloc.cu",
              "cf_adjoint.cu"]
CPP_SOURCES = ["cf_mesh.cpp", "cf_api.cpp", "cf_adjoint_api.cpp", "cf_io.cpp", "cf_cgns.cpp"]
HEADERS = ["cf_internal.h", "cf_flux.h", "cf_dual.h", "cf_ctx.h", "cf_xd.h", "cf_edge_kernel.cuh"]


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES + HEADERS] + [
        os.path.join(ROOT, "include", "cuteflow_gb300.h"), os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA_HOME, "include")]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        # -fmad=false: no FMA contraction, so the kernels round exactly like the reference's
        # sequence of FP64 operations (see csrc/cf_flux.h)
        jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                                     "-diag-suppress", "1444", "-Xcompiler", "-Wno-deprecated-declarations",
                                     "-c", os.path.join(CSRC, s), "-o", o] + inc)
    for s in CPP_SOURCES:
        o = os.path.join(BUILD, s + ".o")
        objs.append(o)
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                     "-Wno-deprecated-declarations", "-c", os.path.join(CSRC, s), "-o", o] + inc)
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    failed = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(j))
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    link = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

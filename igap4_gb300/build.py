"""Build libigapgpu.so in-tree with nvcc for sm_103a (GB300).

Usage:  python -m igap4_gb300.build     (or igap4_gb300.build.build())

Each CUDA translation unit is compiled in parallel, then linked with the host
C sources of the IGAP4-facing layer.  Outputs land next to this file and are
git-ignored; nothing is installed into site-packages.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libigapgpu.so")

CU_SOURCES = ["context.cu", "assemble.cu", "krylov.cu", "noalloc.cu", "tc_tangent.cu", "graph.cu", "predictor.cu",
              "batch.cu", "tc_gram.cu", "tc_ozaki.cu", "density.cu", "cubic.cu", "res_df.cu"]
C_SOURCES: list[str] = []
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-warn-spills"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "igapgpu.h"))
    newest_header = max(os.path.getmtime(h) for h in headers)
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_header):
            jobs.append([nvcc, *ARCH, *NVFLAGS, *inc, "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".c.o"))
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_header):
            jobs.append(["gcc", "-O2", "-std=c99", "-fPIC", "-Wall", *inc,
                         "-I", "/usr/local/cuda/include", "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for out in outs:
                if out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

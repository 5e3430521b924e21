"""Build libjurassic_gb300.so in-tree with nvcc for sm_103a (GB300).

Each CUDA translation unit is compiled in parallel; the FP64 unit without
FMA contraction (rounding like the reference), the mixed unit with it.  The
continuum coefficient tables (data/continua.bin) are embedded as a generated
source file.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libjurassic_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
UNITS = {
    "jgb_fp64.cu": ["-fmad=false"],
    "jgb_mixed.cu": ["-prec-div=false", "-ftz=true"],
    "jgb_api.cu": [],
    "jgb_noalloc.cu": [],
    "jgb_normal.cu": ["-fmad=false"],
    "jgb_retrieval.cu": ["-fmad=false"],
    "jgb_tblio.cu": [],
    # FP32 increments around an FP64 position and direction: approximate
    # FP32 division and square root (~2 ulp) cut the latency of a step
    "jgb_trace_mixed.cu": ["-fmad=false", "-prec-div=false", "-prec-sqrt=false"],
}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _continua_source(path):
    blob = np.fromfile(os.path.join(PKG, "data", "continua.bin"), dtype="<f8")
    with open(path, "w") as f:
        f.write("/* generated from data/continua.bin by build.py */\n")
        f.write("const long jgb_continua_count = %d;\n" % len(blob))
        f.write("const double jgb_continua_blob[%d] = {\n" % len(blob))
        for i in range(0, len(blob), 4):
            f.write("  " + ", ".join("%.17g" % v for v in blob[i:i + 4]) + ",\n")
        f.write("};\n")


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", "jurassic_gb300.h"), os.path.join(PKG, "data", "continua.bin"),
              os.path.abspath(__file__)]
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def build(force=False, verbose=False, extra=()):
    """Compile the library if sources are newer than the built .so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    ctm = os.path.join(BUILD, "jgb_continua_data.c")
    _continua_source(ctm)
    jobs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        jobs.append([cc] + COMMON + flags + list(extra) + ["-c", os.path.join(CSRC, unit), "-o", obj])
    ctm_obj = os.path.join(BUILD, "jgb_continua_data.o")
    jobs.append(["gcc", "-O2", "-fPIC", "-c", ctm, "-o", ctm_obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stderr or r.stdout):
            print(r.stdout + r.stderr, file=sys.stderr)
        return r

    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, u.replace(".cu", ".o")) for u in UNITS] + [ctm_obj]
    tmp = LIB + ".%d.tmp" % os.getpid()
    run([cc] + ARCH + ["-shared", "-Xlinker", "--no-undefined", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)

"""Build libghmm.so in-tree: CUDA kernels for sm_103a plus the C++ host runtime, in parallel.

    python -m gatk_gb300.build [--force] [--verbose]

The library lands in gatk_gb300/_lib/libghmm.so (git-ignored) and links the CUDA runtime
statically, so it loads with only the driver present.  The synthetic workload generator
(include/ghmm_synth.h) is input generation for tests and benchmarks, not part of the product: it is
built beside it as gatk_gb300/_lib/libghmm_synth.so, host code only.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libghmm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kernels.cu", "noalloc.cu", "calib.cu", "post.cu", "pd.cu", "pd_packed.cu", "prep.cu", "sw.cu"]
CPP_SOURCES = ["runtime.cpp", "batch.cpp", "queue.cpp", "pd_host.cpp", "raw_host.cpp", "tables.cpp", "str_analyzer.cpp",
               "sw_host.cpp", "multi.cpp"]
SYNTH_SOURCES = ["synth.cpp"]
SYNTH_LIB = os.path.join(OUT_DIR, "libghmm_synth.so")
HEADERS = ["fp32_rows.cuh", "ghmm_internal.h", "runtime_internal.h", "tables.h", "str_analyzer.h", "host_util.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gatk_gb300")


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES + SYNTH_SOURCES]


def _deps():
    return _sources() + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE) if h.endswith(".h")] + [os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not (os.path.exists(LIB) and os.path.exists(SYNTH_LIB)):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(SYNTH_LIB))
    return all(os.path.getmtime(d) <= t for d in _deps() if os.path.exists(d))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    jobs = []
    for s in CU_SOURCES:
        obj = os.path.join(OBJ_DIR, s + ".o")
        cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-c",
               os.path.join(CSRC, s), "-o", obj]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, obj))
    for s in CPP_SOURCES:
        obj = os.path.join(OBJ_DIR, s + ".o")
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
               "-fno-fast-math", "-Wall", "-I", INCLUDE, "-I", cuda_include(), "-c", os.path.join(CSRC, s), "-o", obj]
        jobs.append((cmd, obj))
    synth_tmp = SYNTH_LIB + ".tmp"
    synth_job = ([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
                  "-fno-fast-math", "-Wall", "-shared", "-I", INCLUDE, *[os.path.join(CSRC, x) for x in SYNTH_SOURCES],
                  "-o", synth_tmp], synth_tmp)
    with ThreadPoolExecutor(max_workers=len(jobs) + 1) as ex:
        logs = list(ex.map(lambda j: _run(j[0], verbose), jobs + [synth_job]))
    os.replace(synth_tmp, SYNTH_LIB)
    if ptxas_verbose:
        print("\n".join(logs))
    tmp = LIB + ".tmp"
    _run([nv, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *[o for _, o in jobs], "-lpthread", "-ldl"], verbose)
    os.replace(tmp, LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print ptxas register/spill report")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose=a.verbose, ptxas_verbose=a.ptxas))


if __name__ == "__main__":
    main(sys.argv[1:])

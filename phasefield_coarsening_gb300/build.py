"""Build recipe: compiles the CUDA library, the `ppf` driver and the oracle.

Outputs (all git-ignored, in-tree):
  phasefield_coarsening_gb300/_build/libppf_gb300.so   C-ABI (include/ppf.h, include/ppf_h5.h)
  phasefield_coarsening_gb300/_build/ppf               drop-in for the reference's `ppf`
  oracle/_build/libppf_oracle.so                       CPU restatement + the oracle's own HDF5
                                                       subset (test infrastructure)

sm_103a only: every .cu file is compiled with
  -gencode arch=compute_103a,code=sm_103a -lineinfo
Translation units compile in parallel; a unit is rebuilt only when a source
or header it may include is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")
ORACLE = os.path.join(REPO, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
                     "--expt-relaxed-constexpr"]

LIB = os.path.join(BUILD, "libppf_gb300.so")
EXE = os.path.join(BUILD, "ppf")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "libppf_oracle.so")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max(os.path.getmtime(p) for p in paths)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-6000:])
    return r.stdout + r.stderr


def _stale(out: str, deps) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < _newest(deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for cu in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(cu)[:-3] + ".o")
        objs.append(obj)
        if ptxas_info or _stale(obj, [cu] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", cu, "-o", obj])
    for c in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        if os.path.basename(c) == "ppf_main.c":
            continue
        obj = os.path.join(BUILD, os.path.basename(c)[:-2] + "_c.o")
        objs.append(obj)
        if _stale(obj, [c] + hdrs):
            jobs.append(["gcc", "-std=c99", "-O2", "-fPIC", "-Wall", "-I", INCLUDE, "-c", c, "-o", obj])
    oracle_src = os.path.join(ORACLE, "ppf_oracle.c")
    shim = os.path.join(ORACLE, "hdf5_shim")
    h5ref = os.path.join(shim, "h5ref.c")
    if _stale(ORACLE_LIB, [oracle_src, h5ref, os.path.join(shim, "h5ref.h"), os.path.join(ORACLE, "ppf_oracle.h"),
                           os.path.join(INCLUDE, "ppf.h")]):
        jobs.append(["gcc", "-std=c99", "-O2", "-fopenmp", "-fPIC", "-shared", "-I", INCLUDE, "-I", shim, oracle_src,
                     h5ref, "-o", ORACLE_LIB, "-lm"])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs)
        os.replace(LIB + ".tmp", LIB)
    main_c = os.path.join(CSRC, "ppf_main.c")
    if os.path.exists(main_c) and _stale(EXE, [main_c, LIB] + hdrs):
        _run(["gcc", "-std=c99", "-O2", "-Wall", "-I", INCLUDE, main_c, "-o", EXE, "-L", BUILD, "-lppf_gb300",
              "-Wl,-rpath,$ORIGIN", "-lm"])
    log = "\n".join(l for l in logs if l.strip())
    if verbose and log:
        print(log)
    return {"lib": LIB, "exe": EXE, "oracle": ORACLE_LIB, "log": log}


if __name__ == "__main__":
    info = build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(info["lib"])

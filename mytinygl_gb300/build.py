"""Build recipe of libmytinygl_gb300.so: the C99 GL front end plus the sm_103a CUDA back end.

Front end: gcc -O2 -ffp-contract=off (the reference's float order, no FMA contraction).
Kernels:   nvcc for sm_103a only, -fmad=false with IEEE division and square root, so every
           float operation rounds as the reference's does on x86-64.
Translation units compile in parallel; an object is rebuilt when any source or header is
newer. The library is built in-tree (mytinygl_gb300/lib/) and links the CUDA runtime
statically. build(debug_bounds=True) builds libmytinygl_gb300_debug.so instead, with
MTGL_DEBUG_BOUNDS defined: the kernels check the indices of their data-dependent accesses
and record a failing site in mtgl_stats.debug_status instead of making the access.
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
INCLUDE = os.path.join(REPO, "include")
FRONT_DIR = os.path.join(PKG, "csrc", "front")
DEV_DIR = os.path.join(PKG, "csrc", "dev")
SERVE_DIR = os.path.join(PKG, "csrc", "serve")
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libmytinygl_gb300.so")
DEBUG_OBJ_DIR = os.path.join(LIB_DIR, "obj_debug")
DEBUG_LIB_PATH = os.path.join(LIB_DIR, "libmytinygl_gb300_debug.so")
EXPORTS = os.path.join(PKG, "csrc", "exports.map")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-ftz=false", "-Xcompiler", "-fPIC", "-Xptxas", "-v", f"-I{INCLUDE}", f"-I{DEV_DIR}"]
CC_FLAGS = ["-O2", "-std=gnu99", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-Wall", f"-I{INCLUDE}"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 back end cannot be built")


def _headers():
    hs = glob.glob(os.path.join(INCLUDE, "*", "*.h"))
    hs += glob.glob(os.path.join(FRONT_DIR, "*.h")) + glob.glob(os.path.join(DEV_DIR, "*.h"))
    hs += glob.glob(os.path.join(DEV_DIR, "*.cuh")) + [EXPORTS, os.path.abspath(__file__)]
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(f) > t for f in [src] + headers)


def _run(cmd, log):
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}{r.stderr}")
    return r


def build(verbose=False, force=False, debug_bounds=False) -> str:
    obj_dir, lib_path = (DEBUG_OBJ_DIR, DEBUG_LIB_PATH) if debug_bounds else (OBJ_DIR, LIB_PATH)
    extra = ["-DMTGL_DEBUG_BOUNDS"] if debug_bounds else []
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = nvcc_path()
    headers = _headers()
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(DEV_DIR, "*.cu"))):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(FRONT_DIR, "*.c")) + glob.glob(os.path.join(SERVE_DIR, "*.c"))):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append(["gcc"] + CC_FLAGS + extra + ["-pthread", "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, j, j[-1] + ".log") for j in jobs]
            for f in futs:
                f.result()
    if force or jobs or not os.path.exists(lib_path):
        tmp = lib_path + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs +
             ["-Xlinker", "-Bsymbolic", "-Xlinker", "--exclude-libs,ALL", "-Xlinker",
              f"--version-script={EXPORTS}", "-lm", "-lpthread"], os.path.join(obj_dir, "link.log"))
        os.replace(tmp, lib_path)
    if verbose:
        print(f"built {lib_path} ({len(jobs)} objects rebuilt)")
    return lib_path


def ptxas_report() -> str:
    """Registers / spills / shared memory per kernel from the last build's -Xptxas -v logs."""
    out = []
    for log in sorted(glob.glob(os.path.join(OBJ_DIR, "*.cu.o.log"))):
        for line in open(log):
            if "ptxas info" in line and ("registers" in line or "Compiling entry" in line or "spill" in line):
                out.append(line.rstrip())
    return "\n".join(out)


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    if "--ptxas" in sys.argv:
        print(ptxas_report())

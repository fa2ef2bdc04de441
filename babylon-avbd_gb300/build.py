"""Build the engine's shared library ``avbd_gb300/libavbd_gb300.so`` for sm_103a.

Each CUDA translation unit is compiled in parallel with nvcc (one ``-gencode``), then linked
with ``-shared``. The collision, solve, engine, sleep and event units are compiled with ``-fmad=false`` so their
float arithmetic is rounded operation by operation, as the reference's is.

Usage: python babylon-avbd_gb300/build.py [--force]   (AVBD_DEFINES="NAME=VALUE ..." adds -D flags)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "avbd_gb300")
LIB = os.path.join(OUT_DIR, "libavbd_gb300.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
UNITS = {
    "scan.cu": [],
    "collide.cu": ["-fmad=false"],
    "solve.cu": ["-fmad=false"],
    "engine.cu": ["-fmad=false"],
    "server.cu": [],
    "bvh.cu": [],
    "sleep.cu": ["-fmad=false"],
    "events.cu": ["-fmad=false"],
    "queries.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for name in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, name)) > t:
            return True
    hdr = os.path.join(os.path.dirname(HERE), "include", "avbd_gb300.h")
    return os.path.getmtime(hdr) > t or os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _sources_newer(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    # extra -D definitions (tuning parameters of the kernels, e.g. AVBD_PRIMAL_TILE=512)
    defines = ["-D" + d for d in os.environ.get("AVBD_DEFINES", "").split()]

    def compile_unit(name):
        obj = os.path.join(BUILD, name + ".o")
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], *defines, "-c", os.path.join(CSRC, name), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

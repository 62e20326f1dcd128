"""Builds the C-ABI library libhacc_sr.so in-tree (hacc-coral_gb300/lib/).

Device code is compiled for sm_103a only.  Host code is compiled with
-ffp-contract=off so the tree and list decisions round exactly as the
reference's x86-64 build does.  Translation units compile in parallel.  The
PM kick's transforms link cuFFT from the same toolkit.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libhacc_sr.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhacc_sr.so")


def _flags() -> list[str]:
    return (["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
             "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH)


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _needs(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()
    headers = (glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh"))
               + glob.glob(os.path.join(ROOT, "include", "*.h")))
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            cmd = [nv] + _flags() + ["-c", src, "-o", obj]
            if src.endswith(".cpp"):
                cmd[1:1] = ["-x", "c++"]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg, file=sys.stderr)
    if force or jobs or _needs(LIB, objs):
        cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "lib64")
        cmd = ([nv, "-shared"] + ARCH + ["-Xcompiler", "-fPIC", "-o", LIB] + objs
               + ["-lcufft", "-lpthread", "-Xlinker", "-rpath=" + cudalib])
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

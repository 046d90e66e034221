"""Build librc_gpu.so (CUDA kernels + C ABI + host set-up) for sm_103a, in-tree.

The FP64 path is compiled with --fmad=false and the host code with
-ffp-contract=off: the reference's x86-64 build has no FMA, and contracting
a*b+c would change its rounding.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "librc_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}"]
# translation unit -> extra flags
UNITS = {
    "rc_core.cu": ["--fmad=false"],
    "rc_noalloc.cu": ["--fmad=false"],
    "rc_peak.cu": ["--fmad=false"],
    "rc_chem.cu": ["--fmad=false"],
    "rc_bdf2.cu": ["--fmad=false"],
    "rc_mlp.cu": [],
    # approximate FP32 division/sqrt and FTZ, but no FMA contraction: the FP64
    # Newton update fused into the mixed sweeps must round like rc_core.cu's
    "rc_mixed.cu": ["--ftz=true", "--prec-div=false", "--prec-sqrt=false", "--fmad=false"],
}
HOST_UNITS = ["rc_host.cpp"]


def nvcc() -> str:
    for p in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, u) for u in list(UNITS) + HOST_UNITS] + [
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))
    ] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every unit in parallel and link librc_gpu.so; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    jobs = []
    for unit, extra in UNITS.items():
        obj = os.path.join(BUILD, unit + ".o")
        jobs.append([nv, *ARCH, *NVCC_COMMON, *extra, "-c", os.path.join(CSRC, unit), "-o", obj])
    for unit in HOST_UNITS:
        obj = os.path.join(BUILD, unit + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}",
                     f"-I{os.path.dirname(nv)}/../include", "-c", os.path.join(CSRC, unit), "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out, file=sys.stderr)
    objs = [os.path.join(BUILD, u + ".o") for u in list(UNITS) + HOST_UNITS]
    tmp = LIB + f".tmp{os.getpid()}"
    run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

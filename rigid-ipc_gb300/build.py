"""Build the rigc CUDA library (``_build/librigc.so``) for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library exporting the C ABI of ``include/rigc.h``.  Units whose exact
decisions must match a round-to-nearest restatement bit for bit (broad phase,
constraint set, CCD) are compiled without fused multiply-add contraction;
the barrier, friction and body-energy derivatives allow it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librigc.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = {
    "api.cu": ["--fmad=false"],
    "sort.cu": ["--fmad=false"],
    "barrier.cu": ["--fmad=true"],
    "constraints.cu": ["--fmad=false"],
    "broad_phase.cu": ["--fmad=false"],
    "ccd.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "body.cu": ["--fmad=true"],
    "friction.cu": ["--fmad=true"],
    "step.cu": ["--fmad=false"],
    "autotune.cu": ["--fmad=false"],
    "fp64_peak.cu": ["--fmad=false"],
    "intersect.cu": ["--fmad=false"],
    "pl_ccd.cu": ["--fmad=false"],
}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the rigc CUDA library cannot be built")
    return p


def _compile(unit: str, extra: list, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
    # host code never contracts a*b+c into fma (aarch64 gcc does by default)
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), *extra, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

"""Build libg3lgpu.so (sm_103a) in-tree with nvcc.

Called by __graft_entry__.build() and by the package on import when the
library is missing or older than its sources.  Translation units are compiled
in parallel; the FP64 engine and rule kernels use -fmad=false so that their
products and sums round exactly as the reference's CPU build does.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libg3lgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")

COMMON = ["-std=c++17", "-O3", "-lineinfo", "-I" + CSRC, "-I" + INCLUDE,
          "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
UNITS = {
    "engine.cu": ["-fmad=false"],
    "eval_fp64.cu": ["-fmad=false"],
    "evalmx_k0.cu": ["-fmad=true"],
    "evalmx_k1.cu": ["-fmad=true"],
    "host_api.cu": ["-fmad=false"],
    "probe.cu": ["-fmad=true"],
    "precompute.cu": ["-fmad=false"],
}
HOST_UNITS = ["host_cubature.cpp", "host_model.cpp", "host_io.cpp"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(INCLUDE, "*.h")))


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for src, extra in UNITS.items():
        obj = os.path.join(OUT, src + ".o")
        jobs.append([NVCC] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj])
    for src in HOST_UNITS:
        obj = os.path.join(OUT, src + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I" + CSRC,
                     "-I" + INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            if l:
                print(l)
    objs = [os.path.join(OUT, s + ".o") for s in list(UNITS) + HOST_UNITS]
    tmp = LIB + ".tmp%d" % os.getpid()
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))

"""In-tree build of libcorr_gb300.so (sm_103a) with nvcc.

Each translation unit under csrc/ is compiled in parallel into
corr_gb300/_build/, then linked into corr_gb300/libcorr_gb300.so.  Only
compute_103a/sm_103a code is generated.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcorr_gb300.so")
SHIM_SRC = os.path.join(PKG, "shim", "corr_shim.cc")
SHIM_LIB = os.path.join(PKG, "libcorr_shim.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _needs(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _needs(obj, [src] + headers) or ptxas_info:
            cmd = [NVCC] + ARCH + FLAGS + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or ptxas_info or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    failed.append(cmd[-3])
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(failed))
    if jobs or not os.path.exists(LIB) or _needs(LIB, objs):
        # the driver API (cuTensorMapEncodeTiled) is resolved at run time through
        # cudaGetDriverEntryPointByVersion, so the library loads without libcuda
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    build_shim()
    return LIB


def build_shim():
    """The drop-in C++ layer (reference signatures) over libcorr_gb300.so."""
    deps = [SHIM_SRC, os.path.join(PKG, "shim", "corr_shim.h"), LIB]
    if not _needs(SHIM_LIB, deps):
        return SHIM_LIB
    cmd = ["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-o", SHIM_LIB, SHIM_SRC,
           "-L" + PKG, "-lcorr_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("shim build failed:\n" + r.stdout + r.stderr)
    return SHIM_LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)

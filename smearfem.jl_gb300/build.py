"""Build libsmearfem_gpu.so in-tree for sm_103a.

    python smearfem.jl_gb300/build.py [--force] [--verbose]

Each csrc/*.cu translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and linked into
``smearfem.jl_gb300/lib/libsmearfem_gpu.so`` (static CUDA runtime).  Only one
architecture is generated: the library targets GB300 and nothing else.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(OUT_DIR, "libsmearfem_gpu.so")
PROBE_SRC = os.path.join(PKG, "probe", "peaks.cu")
PROBE_LIB = os.path.join(OUT_DIR, "libsfem_probe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fvisibility=hidden"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    objs = [os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    exe = nvcc()

    def compile_one(src, obj):
        if not force and not _stale(obj, [src] + headers):
            return obj, ""
        cmd = [exe, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{p.stderr}")
        return obj, p.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        for obj, log in ex.map(lambda a: compile_one(*a), zip(srcs, objs)):
            if verbose and log:
                print(log, file=sys.stderr)
    if force or _stale(LIB, objs):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stderr}")
        os.replace(tmp, LIB)
    if force or _stale(PROBE_LIB, [PROBE_SRC]):
        tmp = PROBE_LIB + f".{os.getpid()}.tmp"
        cmd = [exe, *ARCH, *NVCC_FLAGS, "-shared", "-o", tmp, PROBE_SRC]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"probe build failed:\n{p.stderr}")
        os.replace(tmp, PROBE_LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true", help="print register/spill usage")
    a = ap.parse_args()
    extra = ("-Xptxas", "-v") if a.ptxas_v else ()
    print(build(force=a.force or a.ptxas_v, verbose=a.verbose or a.ptxas_v, extra_flags=extra))

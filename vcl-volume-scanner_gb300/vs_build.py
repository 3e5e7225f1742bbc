"""Builds the package's native libraries in-tree.

* libvs_gb300.so  -- CUDA kernels + C++ host layer + C ABI (include/vs.h),
  sm_103a only, every translation unit compiled in parallel with -fmad=false
  (see csrc/vs_internal.cuh for the arithmetic contract).
* libvs_synth.so  -- host-only synthetic depth generator (csrc/vs_synth.h).

Objects go to _build/ beside this file; the libraries sit beside this file.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")

CU_SOURCES = [
    "k_filter.cu", "k_icp.cu", "k_integrate.cu", "k_raycast.cu", "k_mesh.cu", "vs_api.cu", "vs_batch.cu",
    "vs_server.cu", "vs_snapshot.cu", "vs_noalloc.cu", "k_register.cu",
]
HEADERS = ["vs_internal.cuh", "vs_host.h"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", CSRC, "-I", os.path.join(ROOT, "include"),
]

LIB = os.path.join(HERE, "libvs_gb300.so")
SYNTH_LIB = os.path.join(HERE, "libvs_synth.so")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "vs.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or _stale(LIB, objs):
        _run([NVCC, "-shared", "-o", LIB] + objs + ["-lcudart", "-Xcompiler", "-pthread"])
    synth_src = os.path.join(CSRC, "synth.cpp")
    if force or _stale(SYNTH_LIB, [synth_src, os.path.join(CSRC, "vs_synth.h")]):
        _run([CXX, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", SYNTH_LIB, synth_src])
    return LIB, SYNTH_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

"""Build recipe for the oracle (test infrastructure only).

* oracle/_build/liboracle.so  -- the C++ restatement (oracle.cpp), always.
* oracle/_ref/libref_pin.so   -- the reference's own _yooji_math_inlines.h
  compiled from the reference tree, only where that tree is present.
* oracle/_ref/libref_pin_cuda.so -- the reference's own _yooji_cuda_math.h
  (per-pixel / per-voxel helpers) compiled as host C++ with the stand-ins of
  oracle/ref_shim/, likewise only where the tree is present.

No -march flags: the same source must build on x86-64 and aarch64.
-ffp-contract=off keeps GCC from fusing multiply-adds (the CUDA side builds
with -fmad=false), so both sides round every operation the same way.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_UTIL = "/root/reference/VCL_Volume_Scanner/STAC/Util"
CXX = os.environ.get("CXX", "g++")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared"]


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_oracle(force=False):
    """OpenMP parallelises the per-pixel / per-sub-cube loops only; every
    result is independent of the thread count (OMP_NUM_THREADS)."""
    out = os.path.join(HERE, "_build", "liboracle.so")
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle.h")]
    if force or not _newer(out, srcs):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call([CXX] + FLAGS + ["-fopenmp", "-o", out, srcs[0]])
    return out


def build_ref_pin(force=False):
    """Returns the path of libref_pin.so, or None when the reference tree is absent."""
    if not os.path.isdir(REF_UTIL):
        return None
    out = os.path.join(HERE, "_ref", "libref_pin.so")
    src = os.path.join(HERE, "ref_pin.cpp")
    hdr = os.path.join(REF_UTIL, "_yooji_math_inlines.h")
    if force or not _newer(out, [src, hdr]):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call([CXX] + FLAGS + ["-fpermissive", "-w", "-I", REF_UTIL, "-o", out, src])
    return out


def build_ref_pin_cuda(force=False):
    """Returns the path of libref_pin_cuda.so, or None when the reference tree is absent."""
    if not os.path.isdir(REF_UTIL):
        return None
    out = os.path.join(HERE, "_ref", "libref_pin_cuda.so")
    src = os.path.join(HERE, "ref_pin_cuda.cpp")
    shim = os.path.join(HERE, "ref_shim")
    deps = [src, os.path.join(shim, "ref_cuda_shim.h"), os.path.join(REF_UTIL, "_yooji_cuda_math.h"),
            os.path.join(REF_UTIL, "_yooji_math_inlines.h")]
    if force or not _newer(out, deps):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call([CXX] + FLAGS + ["-fpermissive", "-w", "-I", shim, "-I", REF_UTIL, "-o", out, src])
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref_pin(force))
    print(build_ref_pin_cuda(force))

"""Build recipe for the oracle (test infrastructure only).

* oracle/_build/liboracle.so  -- the C++ restatement (oracle.cpp), always,
  with the seeded synthetic-input generator (the package's csrc/synth.cpp)
  compiled in, so that a CPU run of the oracle maps no library of the
  package.
* oracle/_ref/libref_pin.so   -- the reference's own _yooji_math_inlines.h
  compiled from the reference tree, only where that tree is present.
* oracle/_ref/libref_pin_cuda.so -- the reference's own _yooji_cuda_math.h
  (per-pixel / per-voxel helpers) compiled as host C++ with the stand-ins of
  oracle/ref_shim/, likewise only where the tree is present.
* oracle/_ref/libref_pin_{render,integ,track,imgproc}.so -- the reference's own
  renderer, integrator, tracker and bilateral-filter sources run as host code
  (see build_ref_pin_gpu), likewise only where the tree is present.
* oracle/_ref/libref_pin_cpu.so -- the pyramid, point / normal map and
  intrinsics functions of the reference's CPU image processor (see
  build_ref_pin_cpu), likewise only where the tree is present.

No -march flags: the same source must build on x86-64 and aarch64.
-ffp-contract=off keeps GCC from fusing multiply-adds (the CUDA side builds
with -fmad=false), so both sides round every operation the same way.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: VS_REFERENCE_ROOT, by default where it is mounted here
REF_ROOT = os.environ.get("VS_REFERENCE_ROOT", "/root/reference")
REF_UTIL = os.path.join(REF_ROOT, "VCL_Volume_Scanner", "STAC", "Util")
SYNTH_DIR = os.path.join(os.path.dirname(HERE), "vcl-volume-scanner_gb300", "csrc")
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
    synth = os.path.join(SYNTH_DIR, "synth.cpp")
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle.h"), synth,
            os.path.join(SYNTH_DIR, "vs_synth.h")]
    if force or not _newer(out, srcs):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        subprocess.check_call([CXX] + FLAGS + ["-fopenmp", "-pthread", "-I", SYNTH_DIR, "-o", out, srcs[0], synth])
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


REF_STAC = os.path.dirname(REF_UTIL)
# kernel launches `k<<<grid, block>>>(` -> the host launch loop of the shim
_LAUNCH = r"(\w+)\s*<<<([^<>]*)>>>\s*\("
_GPU_SOURCES = {"math": "Util/z_yooji_cuda_math.cu", "renderer": "Engine/GPU/z_yooji_cuda_tsdf_renderer.cu",
                "integrator": "Engine/GPU/z_yooji_cuda_volume_integrator.cu",
                "tracker": "Engine/GPU/z_yooji_cuda_pose_tracker.cu", "imgproc": "Engine/GPU/z_yooji_cuda_img_proc.cu"}


def build_ref_pin_gpu(force=False):
    """The reference's renderer, integrator, tracker and bilateral filter run
    as host code.  Returns {"render", "integ", "track", "imgproc": path}, or
    None when the reference tree is absent.

    The launch syntax is the only text changed: each source is read from the
    reference tree, its `<<<...>>>` launches are turned into calls of the host
    launch loop, and the result is written to oracle/_ref/gen/ (a build
    product, never committed) and compiled with oracle/ref_pin_gpu.cpp."""
    import re
    if not os.path.isdir(REF_STAC):
        return None
    gen = os.path.join(HERE, "_ref", "gen")
    shim = os.path.join(HERE, "ref_shim", "gpu")
    outs = {"render": os.path.join(HERE, "_ref", "libref_pin_render.so"),
            "integ": os.path.join(HERE, "_ref", "libref_pin_integ.so"),
            "track": os.path.join(HERE, "_ref", "libref_pin_track.so"),
            "imgproc": os.path.join(HERE, "_ref", "libref_pin_imgproc.so")}
    srcs = [os.path.join(REF_STAC, v) for v in _GPU_SOURCES.values()]
    deps = srcs + [os.path.join(HERE, f) for f in ("ref_pin_gpu.cpp", "ref_gpu_runtime.cpp")] + \
        [os.path.join(shim, f) for f in os.listdir(shim)]
    if not force and all(_newer(o, deps) for o in outs.values()):
        return outs
    os.makedirs(gen, exist_ok=True)
    pat = re.compile(_LAUNCH)
    for name, rel in _GPU_SOURCES.items():
        with open(os.path.join(REF_STAC, rel), encoding="latin-1") as f:
            text = f.read()
        text = pat.sub(lambda m: "vs_launch_any(%s, [&](auto&&... vs_a) { %s(vs_a...); })(" % (m.group(2), m.group(1)),
                       text)
        with open(os.path.join(gen, name + ".cu.cpp"), "w", encoding="latin-1") as f:
            f.write(text)
        with open(os.path.join(gen, "tu_" + name + ".cpp"), "w") as f:
            f.write('#include "ref_gpu_shim.h"\n#include "%s.cu.cpp"\n' % name)
    inc = ["-I", shim, "-I", os.path.join(REF_STAC, "Engine", "GPU"), "-I", REF_UTIL, "-I", gen]
    cflags = ["-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-fpermissive", "-w"]
    objs = {}
    for name in ("math",):
        objs[name] = os.path.join(gen, name + ".o")
        subprocess.check_call([CXX] + cflags + inc + ["-c", "-x", "c++", os.path.join(gen, "tu_" + name + ".cpp"),
                               "-o", objs[name]])
    objs["rt"] = os.path.join(gen, "rt.o")
    subprocess.check_call([CXX] + cflags + ["-I", shim, "-c", os.path.join(HERE, "ref_gpu_runtime.cpp"), "-o", objs["rt"]])
    for key, macro in (("render", "REF_PIN_RENDER"), ("integ", "REF_PIN_INTEG"), ("track", "REF_PIN_TRACK"),
                       ("imgproc", "REF_PIN_IMGPROC")):
        o = os.path.join(gen, key + ".o")
        subprocess.check_call([CXX] + cflags + inc + ["-D" + macro, "-c", "-x", "c++",
                               os.path.join(HERE, "ref_pin_gpu.cpp"), "-o", o])
        subprocess.check_call([CXX, "-shared", "-o", outs[key], o, objs["math"], objs["rt"]])
    # the rewritten sources and objects are intermediate: keep only the libraries
    for f in os.listdir(gen):
        os.remove(os.path.join(gen, f))
    os.rmdir(gen)
    return outs


# member functions taken from the reference's CPU sources: (file, qualified
# name, text that must follow the opening parenthesis, for overloads)
_CPU_FUNCTIONS = [
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Intrinsics::set_from_params", ""),
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Intrinsics::get_params", ""),
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Intrinsics::back_project", "CKvPixel"),
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Intrinsics::back_project", "CKvPointf"),
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Intrinsics::project", ""),
    ("Object/CPU/z_yooji_camera_parameters.cpp", "CKvYooji_Extrinsics::transform", ""),
    ("Object/CPU/z_yooji_matrix_rgbd.cpp", "CKvYooji_MatrixRgbD::convert_pixel_coord", ""),
    ("Engine/CPU/z_yooji_object_scanner.cpp",
     "CKvYooji_3D_Object_Scanner::z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates", ""),
    ("Object/CPU/z_yooji_image_pyramid.cpp", "CKvYooji_Pyramid_Mat_Float::c_Create", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::cpm_Compute_Point_Map", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::enm_Estimate_Normal_Map", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::cpdd_Construct_Pyramids_Down_Depth", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::sdg5_Smooth_Depthmap_Gaussian_5x5", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::ddh_Downsample_Depthmap_Half", ""),
    ("Engine/CPU/z_yooji_image_processor.cpp", "LCKvYooji_Image_Processor::dih_Downsample_Intrinsics_Half", ""),
]


def _skip_to(text, i, targets):
    """index of the first character in `targets` at or after i outside
    comments and string / character literals"""
    n = len(text)
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            i = text.find("\n", i)
            i = n if i < 0 else i
        elif text.startswith("/*", i):
            i = text.find("*/", i + 2)
            i = n if i < 0 else i + 2
            continue
        elif c in "\"'":
            j = i + 1
            while j < n and text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j
        elif c in targets:
            return i
        i += 1
    raise ValueError("unbalanced source")


def _function_text(text, qualname, after):
    """the definition of qualname (return type to closing brace)"""
    import re
    pat = re.compile(r"(^|\n)([ \t]*[\w:<>\*& \t]+?\b)" + re.escape(qualname) + r"\s*\(\s*" + re.escape(after))
    for m in pat.finditer(text):
        start = m.start(2)
        i = text.index("(", m.end(2) + len(qualname))
        depth = 0
        while True:  # the parameter list
            i = _skip_to(text, i, "()")
            depth += 1 if text[i] == "(" else -1
            i += 1
            if depth == 0:
                break
        j = _skip_to(text, i, "{;")
        if text[j] == ";":
            continue  # a declaration
        depth = 0
        while True:  # the body
            j = _skip_to(text, j, "{}")
            depth += 1 if text[j] == "{" else -1
            j += 1
            if depth == 0:
                return text[start:j]
    raise ValueError("%s not found" % qualname)


def build_ref_pin_cpu(force=False):
    """Member functions of the reference's CPU image processor, intrinsics and
    pyramid classes, copied unchanged from the reference tree into
    oracle/_ref/gen/cpu_functions.cpp and compiled with oracle/ref_pin_cpu.cpp
    over the KAISION stand-ins.  Returns the path of libref_pin_cpu.so, or
    None when the reference tree is absent."""
    if not os.path.isdir(REF_STAC):
        return None
    out = os.path.join(HERE, "_ref", "libref_pin_cpu.so")
    shim = os.path.join(HERE, "ref_shim", "cpu")
    srcs = sorted({os.path.join(REF_STAC, f) for f, _, _ in _CPU_FUNCTIONS})
    deps = srcs + [os.path.join(HERE, "ref_pin_cpu.cpp"), os.path.join(shim, "ref_kaision_shim.h"),
                   os.path.join(REF_UTIL, "_yooji_SITM_defines.h")]
    if not force and _newer(out, deps):
        return out
    gen = os.path.join(HERE, "_ref", "gen_cpu")
    os.makedirs(gen, exist_ok=True)
    texts = {}
    parts = []
    for f, name, after in _CPU_FUNCTIONS:
        if f not in texts:
            with open(os.path.join(REF_STAC, f), encoding="latin-1") as fh:
                texts[f] = fh.read()
        parts.append("// %s: %s\n%s\n" % (f, name, _function_text(texts[f], name, after)))
    with open(os.path.join(gen, "cpu_functions.cpp"), "w", encoding="latin-1") as fh:
        fh.write("\n".join(parts))
    subprocess.check_call([CXX] + FLAGS + ["-fpermissive", "-w", "-I", shim, "-I", gen, "-I", REF_UTIL, "-o", out,
                                           os.path.join(HERE, "ref_pin_cpu.cpp")])
    os.remove(os.path.join(gen, "cpu_functions.cpp"))
    os.rmdir(gen)
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref_pin(force))
    print(build_ref_pin_cuda(force))
    print(build_ref_pin_gpu(force))
    print(build_ref_pin_cpu(force))

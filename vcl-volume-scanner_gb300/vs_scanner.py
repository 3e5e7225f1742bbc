"""Python binding of the GB300 reconstruction core (ctypes over include/vs.h).

The classes mirror the reference's per-frame interface
(VCL_Volume_Scanner/STAC/Engine/GPU/_yooji_cuda_*.h and so_Scan_Object in
STAC/Engine/CPU/z_yooji_object_scanner.cpp): a ``Session`` carries what
``ip_Initialize_Parameters`` configured, and exposes
``bfd_bilateral_filter_depth``, ``tp_track_pose``,
``cdtoc_convert_depth_to_tsdf``, ``rmi_render_maps_for_icp`` and the fused
``scan_frame``.  Device pointers are passed as integers (for example
``torch.Tensor.data_ptr()``); host arrays are numpy arrays.

The library must be built (``build.py``) and a CUDA device present: there is
no CPU fallback, and every compute call raises ``VsError`` otherwise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvs_gb300.so")
SYNTH_PATH = os.path.join(HERE, "libvs_synth.so")

VS_OK = 0
VS_ERR_ARG = -1
VS_ERR_CUDA = -2
VS_ERR_STATE = -3
VS_ERR_MEMORY = -4

VS_TSDF_INT16, VS_TSDF_FP16, VS_TSDF_FP32 = 0, 1, 2
VS_REDUCE_FP32, VS_REDUCE_KAHAN, VS_REDUCE_FP64 = 0, 1, 2


class VsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("vs error %d: %s" % (code, msg))
        self.code = code


class VsConfig(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float), ("cy", ctypes.c_float),
        ("levels", ctypes.c_int),
        ("dim", ctypes.c_int * 3),
        ("origin", ctypes.c_float * 3),
        ("voxel_size", ctypes.c_float),
        ("mu", ctypes.c_float),
        ("max_w", ctypes.c_float),
        ("th_icp", ctypes.c_float),
        ("cos_normal", ctypes.c_float),
        ("icp_iters", ctypes.c_int * 3),
        ("reduce_mode", ctypes.c_int),
        ("tsdf_type", ctypes.c_int),
        ("depth_scale", ctypes.c_float),
    ]


class SynthConfig(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("fx", ctypes.c_float), ("fy", ctypes.c_float), ("cx", ctypes.c_float), ("cy", ctypes.c_float),
        ("n_frames", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("orbit_radius", ctypes.c_double),
        ("view_distance", ctypes.c_double),
        ("orbit_start_deg", ctypes.c_double),
        ("orbit_step_deg", ctypes.c_double),
        ("jitter_deg", ctypes.c_double),
        ("jitter_m", ctypes.c_double),
        ("noise", ctypes.c_int),
        ("dropout_iid", ctypes.c_double),
        ("dropout_blob", ctypes.c_double),
        ("max_depth", ctypes.c_double),
        ("threads", ctypes.c_int),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.POINTER(ctypes.c_float)

# name -> (restype, argtypes)
_SIGS = {
    "vs_config_default": (None, [ctypes.POINTER(VsConfig), _I, _I]),
    "vs_last_error": (ctypes.c_char_p, []),
    "vs_device_count": (_I, []),
    "vs_session_create": (_I, [ctypes.POINTER(VsConfig), ctypes.POINTER(_P)]),
    "vs_session_destroy": (_I, [_P]),
    "vs_session_reset": (_I, [_P]),
    "vs_session_bytes": (ctypes.c_size_t, [ctypes.POINTER(VsConfig)]),
    "vs_bilateral_filter_depth": (_I, [_P, _P, _P, _I, _I]),
    "vs_bilateral_filter_depth_host": (_I, [_P, _P, _P, _I, _I]),
    "vs_track_pose": (_I, [_P, _P, ctypes.POINTER(_I)]),
    "vs_integrate_depth": (_I, [_P, _P, _I, _I, _P, _P]),
    "vs_render_maps": (_I, [_P, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P]),
    "vs_scan_frame": (_I, [_P, _P, _P]),
    "vs_scan_frame_host": (_I, [_P, _P, _P, ctypes.POINTER(_I)]),
    "vs_session_sync": (_I, [_P]),
    "vs_stage_filter": (_I, [_P, _P]),
    "vs_stage_track": (_I, [_P]),
    "vs_stage_integrate": (_I, [_P]),
    "vs_stage_raycast": (_I, [_P]),
    "vs_get_pose": (_I, [_P, _P, _P, _P]),
    "vs_set_pose": (_I, [_P, _P]),
    "vs_get_volume": (_I, [_P, _P, _P]),
    "vs_set_volume": (_I, [_P, _P, _P]),
    "vs_get_active_bricks": (_I, [_P, ctypes.POINTER(ctypes.c_uint32), _P, ctypes.c_uint32]),
    "vs_get_maps": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "vs_set_stage_timing": (_I, [_P, _I]),
    "vs_get_stage_times": (_I, [_P, _P]),
    "vs_get_frame_stats": (_I, [_P, _P]),
    "vs_kernels_per_frame": (_I, [ctypes.POINTER(VsConfig)]),
    "vs_get_input_raw": (_I, [_P, _P]),
    "vs_get_device_buffer": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "vs_integrate_depth_noalloc": (_I, [_P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P, _I, _I, _P,
                                        _P, _P, _P]),
}

_lib = None
_synth = None


def load(path=LIB_PATH):
    """Loads libvs_gb300.so (raises OSError when it is missing)."""
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def load_synth(path=SYNTH_PATH):
    global _synth
    if _synth is None:
        lib = ctypes.CDLL(path)
        lib.vs_synth_default.restype = None
        lib.vs_synth_default.argtypes = [ctypes.POINTER(SynthConfig), _I, _I]
        lib.vs_synth_generate.restype = _I
        lib.vs_synth_generate.argtypes = [ctypes.POINTER(SynthConfig), _P, _P, _P]
        _synth = lib
    return _synth


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc != VS_OK:
        raise VsError(rc, load().vs_last_error().decode())


def default_config(width, height, **kw):
    c = VsConfig()
    load().vs_config_default(ctypes.byref(c), width, height)
    for k, v in kw.items():
        if k in ("dim", "origin", "icp_iters"):
            arr = getattr(c, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(c, k, v)
    return c


def device_count():
    return load().vs_device_count()


def level_intrinsics(cfg):
    """Per-level (W, H, fx, fy, cx, cy) with the reference's halving rule
    (z_yooji_cuda_pose_tracker.cu:764-776), in float32 arithmetic."""
    f32 = np.float32
    fx, fy, px, py = f32(cfg.fx), f32(cfg.fy), f32(cfg.cx), f32(cfg.cy)
    w, h = cfg.width, cfg.height
    out = []
    for _ in range(cfg.levels):
        out.append((w, h, fx, fy, px, py))
        fx, fy = f32(0.5) * fx, f32(0.5) * fy
        px, py = f32(0.5) * (px - f32(0.5)), f32(0.5) * (py - f32(0.5))
        w //= 2
        h //= 2
    return out


class Session:
    """One scanning session: volume, pose, frame pyramid and model maps on the device."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        h = ctypes.c_void_p()
        _check(self.lib.vs_session_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.levels = level_intrinsics(cfg)

    def close(self):
        if self.h:
            self.lib.vs_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- reference-shaped entry points ----
    def bfd_bilateral_filter_depth(self, out_dev, depth_host):
        d = np.ascontiguousarray(depth_host, dtype=np.float32)
        _check(self.lib.vs_bilateral_filter_depth(self.h, _ptr(out_dev), _ptr(d), d.shape[1], d.shape[0]))

    def bfd_bilateral_filter_depth_host(self, depth_host):
        d = np.ascontiguousarray(depth_host, dtype=np.float32)
        out = np.empty_like(d)
        _check(self.lib.vs_bilateral_filter_depth_host(self.h, _ptr(out), _ptr(d), d.shape[1], d.shape[0]))
        return out

    def tp_track_pose(self, init_T01_dev=None):
        t = _I(0)
        _check(self.lib.vs_track_pose(self.h, _ptr(init_T01_dev), ctypes.byref(t)))
        return bool(t.value)

    def cdtoc_convert_depth_to_tsdf(self, depth_dev, T_gc_dev, T_cg_dev):
        _check(self.lib.vs_integrate_depth(self.h, _ptr(depth_dev), self.cfg.width, self.cfg.height,
                                           _ptr(T_gc_dev), _ptr(T_cg_dev)))

    def rmi_render_maps_for_icp(self, level, T_gc_dev, T_cg_dev, cam_cen, light, depth_dev, vertex_dev,
                                normal_dev, img_dev):
        w, h = self.levels[level][0], self.levels[level][1]
        c = np.ascontiguousarray(cam_cen, dtype=np.float32)
        l = np.ascontiguousarray(light, dtype=np.float32)
        _check(self.lib.vs_render_maps(self.h, w, h, _ptr(T_gc_dev), _ptr(T_cg_dev), _ptr(c), _ptr(l), level,
                                       _ptr(depth_dev), _ptr(vertex_dev), _ptr(normal_dev), _ptr(img_dev)))

    # ---- per-frame path ----
    def scan_frame(self, depth_mm_dev, stream=None):
        _check(self.lib.vs_scan_frame(self.h, _ptr(depth_mm_dev), _ptr(stream)))

    def scan_frame_host(self, depth_mm):
        d = np.ascontiguousarray(depth_mm, dtype=np.uint16)
        T = np.empty(16, np.float32)
        t = _I(0)
        _check(self.lib.vs_scan_frame_host(self.h, _ptr(d), _ptr(T), ctypes.byref(t)))
        return T.reshape(4, 4), bool(t.value)

    def sync(self):
        _check(self.lib.vs_session_sync(self.h))

    def reset(self):
        _check(self.lib.vs_session_reset(self.h))

    def stage_filter(self, depth_mm_dev):
        _check(self.lib.vs_stage_filter(self.h, _ptr(depth_mm_dev)))

    def stage_track(self):
        _check(self.lib.vs_stage_track(self.h))

    def stage_integrate(self):
        _check(self.lib.vs_stage_integrate(self.h))

    def stage_raycast(self):
        _check(self.lib.vs_stage_raycast(self.h))

    # ---- state ----
    def pose(self):
        T = np.empty(16, np.float32)
        Td = np.empty(16, np.float64)
        info = np.empty(4, np.int32)
        _check(self.lib.vs_get_pose(self.h, _ptr(T), _ptr(Td), _ptr(info)))
        return T.reshape(4, 4), Td.reshape(4, 4), info

    def set_pose(self, T_gc):
        Td = np.ascontiguousarray(T_gc, dtype=np.float64).reshape(16)
        _check(self.lib.vs_set_pose(self.h, _ptr(Td)))

    def volume(self):
        n = self.cfg.dim[0] * self.cfg.dim[1] * self.cfg.dim[2]
        t = np.empty(n, np.float32)
        w = np.empty(n, np.uint16)
        _check(self.lib.vs_get_volume(self.h, _ptr(t), _ptr(w)))
        return t, w

    def set_volume(self, tsdf, weight):
        t = np.ascontiguousarray(tsdf, dtype=np.float32)
        w = np.ascontiguousarray(weight, dtype=np.uint16)
        _check(self.lib.vs_set_volume(self.h, _ptr(t), _ptr(w)))

    def active_bricks(self):
        c = ctypes.c_uint32(0)
        _check(self.lib.vs_get_active_bricks(self.h, ctypes.byref(c), None, 0))
        out = np.empty(max(1, c.value), np.uint32)
        _check(self.lib.vs_get_active_bricks(self.h, ctypes.byref(c), _ptr(out), out.size))
        return out[: c.value]

    def maps(self, level):
        w, h = self.levels[level][0], self.levels[level][1]
        n = w * h
        md, mv, mn = np.empty(n, np.float32), np.empty(3 * n, np.float32), np.empty(3 * n, np.float32)
        mi = np.empty(n, np.uint8)
        idp, iv, inn = np.empty(n, np.float32), np.empty(3 * n, np.float32), np.empty(3 * n, np.float32)
        _check(self.lib.vs_get_maps(self.h, level, _ptr(md), _ptr(mv), _ptr(mn), _ptr(mi), _ptr(idp), _ptr(iv),
                                    _ptr(inn)))
        return dict(model_depth=md.reshape(h, w), model_vertex=mv.reshape(h, w, 3), model_normal=mn.reshape(h, w, 3),
                    model_img=mi.reshape(h, w), input_depth=idp.reshape(h, w), input_vertex=iv.reshape(h, w, 3),
                    input_normal=inn.reshape(h, w, 3))

    def set_stage_timing(self, enable=True):
        _check(self.lib.vs_set_stage_timing(self.h, 1 if enable else 0))

    def stage_times(self):
        """device ms of the last frame: filter, track, integrate, ray-cast"""
        ms = np.empty(4, np.float32)
        _check(self.lib.vs_get_stage_times(self.h, _ptr(ms)))
        return ms

    def frame_stats(self):
        """active sub-cubes, voxels updated, ICP iterations, correspondences"""
        st = np.empty(4, np.uint32)
        _check(self.lib.vs_get_frame_stats(self.h, _ptr(st)))
        return st

    def kernels_per_frame(self):
        return self.lib.vs_kernels_per_frame(ctypes.byref(self.cfg))

    def input_raw(self):
        out = np.empty((self.cfg.height, self.cfg.width), np.float32)
        _check(self.lib.vs_get_input_raw(self.h, _ptr(out)))
        return out

    def device_buffer(self, which):
        p = ctypes.c_void_p()
        _check(self.lib.vs_get_device_buffer(self.h, which, ctypes.byref(p)))
        return p.value


def synth_config(width, height, **kw):
    c = SynthConfig()
    load_synth().vs_synth_default(ctypes.byref(c), width, height)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def synth_generate(cfg):
    """Returns (depth uint16 [n,h,w], T_gc float64 [n,4,4], scene centre in the global frame)."""
    n, h, w = cfg.n_frames, cfg.height, cfg.width
    depth = np.empty((n, h, w), np.uint16)
    T = np.empty((n, 4, 4), np.float64)
    c = np.empty(3, np.float64)
    rc = load_synth().vs_synth_generate(ctypes.byref(cfg), _ptr(depth), _ptr(T), _ptr(c))
    if rc != 0:
        raise ValueError("bad synth config")
    return depth, T, c


def cube_around(centre, size, dim):
    """origin and voxel size of a dim^3 cube of edge `size` centred on `centre`."""
    vox = np.float32(size) / np.float32(dim)
    origin = np.asarray(centre, np.float64) - size / 2.0
    return [float(x) for x in origin], float(vox)

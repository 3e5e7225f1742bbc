"""Python binding of the GB300 reconstruction core (ctypes over include/vs.h).

The classes mirror the reference's per-frame interface
(VCL_Volume_Scanner/STAC/Engine/GPU/_yooji_cuda_*.h and so_Scan_Object in
STAC/Engine/CPU/z_yooji_object_scanner.cpp): a ``Session`` carries what
``ip_Initialize_Parameters`` configured, and exposes
``bfd_bilateral_filter_depth``, ``tp_track_pose``,
``cdtoc_convert_depth_to_tsdf``, ``rmi_render_maps_for_icp`` and the fused
``scan_frame``.  Device pointers are passed as integers (for example
``torch.Tensor.data_ptr()``); host arrays are numpy arrays.

The library must be built (``vs_build.py``) and a CUDA device present: there is
no CPU fallback, and every compute call raises ``VsError`` otherwise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("VS_LIB", os.path.join(HERE, "libvs_gb300.so"))
SYNTH_PATH = os.path.join(HERE, "libvs_synth.so")

VS_OK = 0
VS_ERR_ARG = -1
VS_ERR_CUDA = -2
VS_ERR_STATE = -3
VS_ERR_MEMORY = -4
VS_ERR_BUSY = -5
VS_MAX_BATCH = 64

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
        ("color", ctypes.c_int),
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


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("hbm_budget", ctypes.c_size_t),
        ("max_resident", ctypes.c_int),
        ("max_batch", ctypes.c_int),
        ("queue_depth", ctypes.c_int),
        ("pipeline", ctypes.c_int),
        ("lanes", ctypes.c_int),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("session", ctypes.c_int), ("frame", ctypes.c_int), ("tracked", ctypes.c_int), ("batch", ctypes.c_int),
        ("T_gc", ctypes.c_float * 16),
        ("t_submit", ctypes.c_double), ("t_done", ctypes.c_double), ("latency_ms", ctypes.c_double),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_uint64), ("frames", ctypes.c_uint64), ("mean_batch", ctypes.c_double),
        ("max_batch_seen", ctypes.c_int), ("resident", ctypes.c_int), ("waiting", ctypes.c_int),
        ("closed", ctypes.c_int), ("bytes_resident", ctypes.c_size_t), ("bytes_budget", ctypes.c_size_t),
    ]


VS_SESSION_WAITING, VS_SESSION_RESIDENT, VS_SESSION_CLOSED = 0, 1, 2

class LaunchShape(ctypes.Structure):
    _fields_ = [("ray_tile_log2", ctypes.c_int), ("march_blocks_per_sm", ctypes.c_int),
                ("shade_blocks_per_sm", ctypes.c_int), ("bilateral_rows", ctypes.c_int),
                ("integrate_blocks_per_sm", ctypes.c_int)]


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
    "vs_get_icp_system": (_I, [_P, _P, _P]),
    "vs_get_band": (_I, [_P, _P, _P]),
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
    "vs_integrate_depth_color": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "vs_render_maps_color": (_I, [_P, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P, _P]),
    "vs_render_maps_scene": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "vs_render_view_scene": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "vs_render_view": (_I, [_P, _I, _I, _P, _P, _P, _P, _I, _P, _P, _P, _P]),
    "vs_update_valid_volume": (_I, [_P, _P, _I, ctypes.POINTER(ctypes.c_uint32)]),
    "vs_set_color_frame": (_I, [_P, _P, _I]),
    "vs_get_color_volume": (_I, [_P, _P]),
    "vs_set_color_volume": (_I, [_P, _P]),
    "vs_get_color_map": (_I, [_P, _I, _P]),
    "vs_session_save": (_I, [_P, ctypes.c_char_p]),
    "vs_session_load": (_I, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "vs_session_config": (_I, [_P, ctypes.POINTER(VsConfig)]),
    "vs_extract_mesh": (_I, [_P, _P, _P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "vs_save_mesh_ply": (_I, [_P, ctypes.c_char_p]),
    "vs_warp_depth_to_color": (_I, [_P, _I, _I, _P, _P, _P, _I, _I, _P, _P]),
    "vs_warp_depth_mm_to_color": (_I, [_P, _I, _I, ctypes.c_float, _P, _P, _P, _I, _I, _P, _P]),
    "vs_integrate_depth_noalloc": (_I, [_P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P, _I, _I, _P,
                                        _P, _P, _P]),
    "vs_batch_create": (_I, [ctypes.POINTER(_P)]),
    "vs_batch_destroy": (_I, [_P]),
    "vs_batch_step": (_I, [_P, _P, _I, _P, _P]),
    "vs_batch_step_host": (_I, [_P, _P, _I, _P, _P, _P]),
    "vs_batch_sync": (_I, [_P]),
    "vs_batch_set_stage_timing": (_I, [_P, _I]),
    "vs_batch_get_stage_times": (_I, [_P, _P]),
    "vs_batch_kernels_per_step": (_I, [_P]),
    "vs_batch_get_launch_shape": (_I, [_P, ctypes.POINTER(LaunchShape)]),
    "vs_batch_set_launch_shape": (_I, [_P, ctypes.POINTER(LaunchShape)]),
    "vs_batch_autotune": (_I, [_P, _P, _I, _I, ctypes.POINTER(LaunchShape), ctypes.POINTER(ctypes.c_float)]),
    "vs_server_config_default": (None, [ctypes.POINTER(ServerConfig)]),
    "vs_server_create": (_I, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "vs_server_destroy": (_I, [_P]),
    "vs_server_open": (_I, [_P, ctypes.POINTER(VsConfig), ctypes.POINTER(_I)]),
    "vs_server_state": (_I, [_P, _I, ctypes.POINTER(_I)]),
    "vs_server_submit": (_I, [_P, _I, _P]),
    "vs_server_close": (_I, [_P, _I]),
    "vs_server_poll": (_I, [_P, ctypes.POINTER(Result), _I, _I]),
    "vs_server_drain": (_I, [_P]),
    "vs_server_get_session": (_I, [_P, _I, ctypes.POINTER(_P)]),
    "vs_server_get_stats": (_I, [_P, ctypes.POINTER(ServerStats)]),
    "vs_server_clock": (ctypes.c_double, []),
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
        lib.vs_synth_generate_rgb.restype = _I
        lib.vs_synth_generate_rgb.argtypes = [ctypes.POINTER(SynthConfig), _P, _P, _P, _P]
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

    def __init__(self, cfg, _handle=None):
        self.lib = load()
        h = ctypes.c_void_p()
        if _handle is None:
            _check(self.lib.vs_session_create(ctypes.byref(cfg), ctypes.byref(h)))
        else:
            h = _handle
            cfg = VsConfig()
            _check(self.lib.vs_session_config(h, ctypes.byref(cfg)))
        self.cfg = cfg
        self.h = h
        self.levels = level_intrinsics(cfg)

    @classmethod
    def load(cls, path):
        """a session resumed from a snapshot written by save()"""
        h = ctypes.c_void_p()
        _check(load().vs_session_load(os.fsencode(path), ctypes.byref(h)))
        return cls(None, _handle=h)

    def save(self, path):
        _check(self.lib.vs_session_save(self.h, os.fsencode(path)))

    def mesh(self, with_color=False):
        """triangle soup of the zero level set: (xyz [n,3,3] float32, rgb [n,3,3] uint8 or None)"""
        n = ctypes.c_uint64(0)
        _check(self.lib.vs_extract_mesh(self.h, None, None, 0, ctypes.byref(n)))
        cap = n.value
        xyz = np.empty((max(cap, 1), 3, 3), np.float32)
        rgb = np.empty((max(cap, 1), 3, 3), np.uint8) if with_color else None
        _check(self.lib.vs_extract_mesh(self.h, _ptr(xyz), _ptr(rgb), cap, ctypes.byref(n)))
        m = min(cap, n.value)
        return xyz[:m], (rgb[:m] if with_color else None)

    def save_mesh_ply(self, path):
        _check(self.lib.vs_save_mesh_ply(self.h, os.fsencode(path)))

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

    def cdtocc_convert_depth_to_tsdf_color(self, depth_dev, rgb_dev, T_gc_dev, T_cg_dev):
        _check(self.lib.vs_integrate_depth_color(self.h, _ptr(depth_dev), _ptr(rgb_dev), self.cfg.width,
                                                 self.cfg.height, _ptr(T_gc_dev), _ptr(T_cg_dev)))

    def rmi_render_maps_color(self, level, T_gc_dev, T_cg_dev, cam_cen, light, depth_dev, vertex_dev, normal_dev,
                              img_dev, rgb_dev):
        w, h = self.levels[level][0], self.levels[level][1]
        c = np.ascontiguousarray(cam_cen, dtype=np.float32)
        l = np.ascontiguousarray(light, dtype=np.float32)
        _check(self.lib.vs_render_maps_color(self.h, w, h, _ptr(T_gc_dev), _ptr(T_cg_dev), _ptr(c), _ptr(l), level,
                                             _ptr(depth_dev), _ptr(vertex_dev), _ptr(normal_dev), _ptr(img_dev),
                                             _ptr(rgb_dev)))

    def rmis_render_maps_for_scene(self, T_gc_dev, T_cg_dev, cam_cen, light, depth_dev, vertex_dev, normal_dev,
                                   img_dev, rgb_dev=None):
        """the scene ray-cast at level 0; vertex_dev None: the form without a
        vertex map (trilinear colour), else the one with it (nearest colour)"""
        w, h = self.levels[0][0], self.levels[0][1]
        c = np.ascontiguousarray(cam_cen, dtype=np.float32)
        l = np.ascontiguousarray(light, dtype=np.float32)
        if vertex_dev is None:
            _check(self.lib.vs_render_view_scene(self.h, w, h, _ptr(T_gc_dev), _ptr(T_cg_dev), _ptr(c), _ptr(l),
                                                 _ptr(depth_dev), _ptr(normal_dev), _ptr(img_dev), _ptr(rgb_dev)))
        else:
            _check(self.lib.vs_render_maps_scene(self.h, w, h, _ptr(T_gc_dev), _ptr(T_cg_dev), _ptr(c), _ptr(l),
                                                 _ptr(depth_dev), _ptr(vertex_dev), _ptr(normal_dev), _ptr(img_dev),
                                                 _ptr(rgb_dev)))

    def rmi_render_view(self, level, T_gc_dev, T_cg_dev, cam_cen, light, depth_dev, normal_dev, img_dev,
                        rgb_dev=None):
        """the object ray-cast without a vertex map: global normals, white background"""
        w, h = self.levels[level][0], self.levels[level][1]
        c = np.ascontiguousarray(cam_cen, dtype=np.float32)
        l = np.ascontiguousarray(light, dtype=np.float32)
        _check(self.lib.vs_render_view(self.h, w, h, _ptr(T_gc_dev), _ptr(T_cg_dev), _ptr(c), _ptr(l), level,
                                       _ptr(depth_dev), _ptr(normal_dev), _ptr(img_dev), _ptr(rgb_dev)))

    def uvv_update_valid_volume(self, valid):
        """valid: host array of dim[0]*dim[1]*dim[2] bytes (x fastest, 0 =
        outside) or an 8-byte aligned device pointer (int); returns the number
        of sub-cubes reset"""
        n = ctypes.c_uint32(0)
        if isinstance(valid, int):
            _check(self.lib.vs_update_valid_volume(self.h, _ptr(valid), 0, ctypes.byref(n)))
        else:
            m = np.ascontiguousarray(valid, dtype=np.uint8).reshape(-1)
            if m.size != self.cfg.dim[0] * self.cfg.dim[1] * self.cfg.dim[2]:
                raise ValueError("valid volume size differs from the session's")
            _check(self.lib.vs_update_valid_volume(self.h, _ptr(m), 1, ctypes.byref(n)))
        return int(n.value)

    def set_color_frame(self, rgb):
        """planar uint8 (3, height, width) host array, or a device pointer (int)"""
        if isinstance(rgb, int):
            _check(self.lib.vs_set_color_frame(self.h, _ptr(rgb), 0))
        else:
            c = np.ascontiguousarray(rgb, dtype=np.uint8)
            _check(self.lib.vs_set_color_frame(self.h, _ptr(c), 1))

    def color_volume(self):
        n = self.cfg.dim[0] * self.cfg.dim[1] * self.cfg.dim[2]
        out = np.empty(3 * n, np.uint8)
        _check(self.lib.vs_get_color_volume(self.h, _ptr(out)))
        return out.reshape(3, n)

    def set_color_volume(self, rgb):
        c = np.ascontiguousarray(rgb, dtype=np.uint8)
        _check(self.lib.vs_set_color_volume(self.h, _ptr(c)))

    def color_map(self, level):
        w, h = self.levels[level][0], self.levels[level][1]
        out = np.empty((3, h, w), np.uint8)
        _check(self.lib.vs_get_color_map(self.h, level, _ptr(out)))
        return out

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

    def icp_system(self):
        """(sums [29] float64, x [6] float32) of the last ICP iteration run"""
        sums = np.empty(29, np.float64)
        x = np.empty(6, np.float32)
        _check(self.lib.vs_get_icp_system(self.h, _ptr(sums), _ptr(x)))
        return sums, x

    def band(self):
        """(band flags, band distances) per sub-cube, shaped (nb_z, nb_y, nb_x)"""
        nb = [self.cfg.dim[k] // 8 for k in range(3)]
        band = np.empty((nb[2], nb[1], nb[0]), np.uint8)
        dist = np.empty((nb[2], nb[1], nb[0]), np.uint8)
        _check(self.lib.vs_get_band(self.h, _ptr(band), _ptr(dist)))
        return band, dist

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


class Batch:
    """Batch runner: advances several sessions by one frame each per step,
    one launch per stage for the whole batch (vs_batch_* in include/vs.h)."""

    def __init__(self):
        self.lib = load()
        h = ctypes.c_void_p()
        _check(self.lib.vs_batch_create(ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.vs_batch_destroy(self.h)
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

    @staticmethod
    def _handles(sessions):
        arr = (ctypes.c_void_p * len(sessions))()
        for i, s in enumerate(sessions):
            arr[i] = s.h.value if isinstance(s.h, ctypes.c_void_p) else s.h
        return arr

    def step(self, sessions, depth_mm_dev=None, stream=None):
        """device frames (integers, or None for frames already in place); returns at once"""
        hs = self._handles(sessions)
        frames = None
        if depth_mm_dev is not None:
            frames = (ctypes.c_void_p * len(sessions))(*[d if d else None for d in depth_mm_dev])
        _check(self.lib.vs_batch_step(self.h, hs, len(sessions), frames, _ptr(stream)))

    def step_host(self, sessions, depth_mm):
        """host uint16 frames in, (T_gc [n,4,4] float32, tracked [n] bool) out"""
        n = len(sessions)
        ds = [np.ascontiguousarray(d, dtype=np.uint16) for d in depth_mm]
        frames = (ctypes.c_void_p * n)(*[d.ctypes.data for d in ds])
        T = np.empty((n, 16), np.float32)
        tr = np.empty(n, np.int32)
        _check(self.lib.vs_batch_step_host(self.h, self._handles(sessions), n, frames, _ptr(T), _ptr(tr)))
        return T.reshape(n, 4, 4), tr.astype(bool)

    def sync(self):
        _check(self.lib.vs_batch_sync(self.h))

    def set_stage_timing(self, enable=True):
        _check(self.lib.vs_batch_set_stage_timing(self.h, 1 if enable else 0))

    def stage_times(self):
        ms = np.empty(4, np.float32)
        _check(self.lib.vs_batch_get_stage_times(self.h, _ptr(ms)))
        return ms

    def kernels_per_step(self):
        return self.lib.vs_batch_kernels_per_step(self.h)

    def launch_shape(self):
        sh = LaunchShape()
        _check(self.lib.vs_batch_get_launch_shape(self.h, ctypes.byref(sh)))
        return (sh.ray_tile_log2, sh.march_blocks_per_sm, sh.shade_blocks_per_sm, sh.bilateral_rows,
                sh.integrate_blocks_per_sm)

    def set_launch_shape(self, ray_tile_log2, march_blocks_per_sm=0, shade_blocks_per_sm=0, bilateral_rows=0,
                         integrate_blocks_per_sm=0):
        sh = LaunchShape(ray_tile_log2, march_blocks_per_sm, shade_blocks_per_sm, bilateral_rows,
                         integrate_blocks_per_sm)
        _check(self.lib.vs_batch_set_launch_shape(self.h, ctypes.byref(sh)))

    def autotune(self, sessions, reps=3):
        """picks the fastest launch shape of the ray-cast, filter and integration
        for these sessions; returns (shape, ray-cast ms)"""
        sh = LaunchShape()
        ms = ctypes.c_float(0.0)
        _check(self.lib.vs_batch_autotune(self.h, self._handles(sessions), len(sessions), reps, ctypes.byref(sh),
                                          ctypes.byref(ms)))
        return (sh.ray_tile_log2, sh.march_blocks_per_sm, sh.shade_blocks_per_sm, sh.bilateral_rows,
                sh.integrate_blocks_per_sm), ms.value


class _Borrowed(Session):
    """a session owned by a server (state access only; never destroyed here)"""

    def __init__(self, handle, cfg):
        self.lib = load()
        self.cfg = cfg
        self.h = ctypes.c_void_p(handle)
        self.levels = level_intrinsics(cfg)

    def close(self):
        self.h = None


class Server:
    """Serving loop: continuous batching of frames from many sessions with
    admission by HBM budget (vs_server_* in include/vs.h)."""

    def __init__(self, hbm_budget=0, max_resident=0, max_batch=0, queue_depth=0, pipeline=0, lanes=0):
        self.lib = load()
        c = ServerConfig()
        self.lib.vs_server_config_default(ctypes.byref(c))
        for k, v in dict(hbm_budget=hbm_budget, max_resident=max_resident, max_batch=max_batch,
                         queue_depth=queue_depth, pipeline=pipeline, lanes=lanes).items():
            if v:
                setattr(c, k, v)
        h = ctypes.c_void_p()
        _check(self.lib.vs_server_create(ctypes.byref(c), ctypes.byref(h)))
        self.h = h
        self.cfgs = {}
        self._buf = (Result * 256)()

    def close(self):
        if self.h:
            self.lib.vs_server_destroy(self.h)
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

    def open(self, cfg):
        i = _I(0)
        _check(self.lib.vs_server_open(self.h, ctypes.byref(cfg), ctypes.byref(i)))
        self.cfgs[i.value] = cfg
        return i.value

    def state(self, sid):
        st = _I(0)
        _check(self.lib.vs_server_state(self.h, sid, ctypes.byref(st)))
        return st.value

    def submit(self, sid, depth_mm):
        """returns False when the session's queue is full"""
        d = np.ascontiguousarray(depth_mm, dtype=np.uint16)
        rc = self.lib.vs_server_submit(self.h, sid, _ptr(d))
        if rc == VS_ERR_BUSY:
            return False
        _check(rc)
        return True

    def close_session(self, sid):
        _check(self.lib.vs_server_close(self.h, sid))

    def poll(self, timeout_ms=0):
        n = self.lib.vs_server_poll(self.h, self._buf, len(self._buf), int(timeout_ms))
        if n < 0:
            _check(n)
        out = []
        for r in self._buf[:n]:
            out.append(dict(session=r.session, frame=r.frame, tracked=bool(r.tracked), batch=r.batch,
                            T_gc=np.array(r.T_gc, np.float32).reshape(4, 4), t_submit=r.t_submit,
                            t_done=r.t_done, latency_ms=r.latency_ms))
        return out

    def drain(self):
        _check(self.lib.vs_server_drain(self.h))

    def session(self, sid):
        p = ctypes.c_void_p()
        _check(self.lib.vs_server_get_session(self.h, sid, ctypes.byref(p)))
        return _Borrowed(p.value, self.cfgs[sid])

    def stats(self):
        st = ServerStats()
        _check(self.lib.vs_server_get_stats(self.h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def clock(self):
        return self.lib.vs_server_clock()


def warp_depth_to_color(depth_dev, w_d, h_d, K_d, T_rgb_wrt_d, K_rgb, w_rgb, h_rgb, out_dev, stream=None, mm_scale=None):
    """depth (device pointer, float metres, or uint16 units when mm_scale is given) seen from the colour camera"""
    kd = np.ascontiguousarray(K_d, np.float32)
    kr = np.ascontiguousarray(K_rgb, np.float32)
    t = np.ascontiguousarray(T_rgb_wrt_d, np.float32).reshape(16)
    lib = load()
    if mm_scale is None:
        _check(lib.vs_warp_depth_to_color(_ptr(depth_dev), w_d, h_d, _ptr(kd), _ptr(t), _ptr(kr), w_rgb, h_rgb,
                                          _ptr(out_dev), _ptr(stream)))
    else:
        _check(lib.vs_warp_depth_mm_to_color(_ptr(depth_dev), w_d, h_d, mm_scale, _ptr(kd), _ptr(t), _ptr(kr), w_rgb,
                                             h_rgb, _ptr(out_dev), _ptr(stream)))


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


def synth_generate_rgb(cfg):
    """(depth uint16 [n,h,w], rgb uint8 [n,3,h,w] planar, T_gc [n,4,4], scene centre)"""
    n, h, w = cfg.n_frames, cfg.height, cfg.width
    depth = np.empty((n, h, w), np.uint16)
    rgb = np.empty((n, 3, h, w), np.uint8)
    T = np.empty((n, 4, 4), np.float64)
    c = np.empty(3, np.float64)
    rc = load_synth().vs_synth_generate_rgb(ctypes.byref(cfg), _ptr(depth), _ptr(rgb), _ptr(T), _ptr(c))
    if rc != 0:
        raise ValueError("bad synth config")
    return depth, rgb, T, c


def cube_around(centre, size, dim):
    """origin and voxel size of a dim^3 cube of edge `size` centred on `centre`."""
    vox = np.float32(size) / np.float32(dim)
    origin = np.asarray(centre, np.float64) - size / 2.0
    return [float(x) for x in origin], float(vox)

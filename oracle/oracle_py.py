"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and the cpu_baseline / reference leg
of bench.py as the checker.  The product never imports this module.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_lib = None
_ref = None

# oracle reduce modes (oracle.h): 0 reference tree, 1 naive fp32, 2 kahan, 3 fp64
ORACLE_REDUCE_FROM_VS = {0: 1, 1: 2, 2: 3}
# oracle tsdf_store: 0 fp32, 1 int16, 2 fp16 ; vs tsdf_type: 0 int16, 1 fp16, 2 fp32
ORACLE_STORE_FROM_VS = {0: 1, 1: 2, 2: 0}
# render variant bits (or_render_variant)
RAY_SCENE, RAY_GLOBAL_NORMALS, RAY_NEAREST_COLOR, RAY_WHITE_BACKGROUND = 1, 2, 4, 8


class OrConfig(ctypes.Structure):
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
        ("tsdf_store", ctypes.c_int),
        ("reduce_mode", ctypes.c_int),
        ("depth_scale", ctypes.c_float),
    ]


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.c_void_p)


def load():
    global _lib
    if _lib is None:
        import build_oracle as _b  # oracle/build_oracle.py (this directory is on sys.path)
        path = _b.build_oracle()
        lib = ctypes.CDLL(path)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        lib.vs_synth_default.restype = None
        lib.vs_synth_default.argtypes = [ctypes.POINTER(SynthConfig), I, I]
        lib.vs_synth_generate.restype = I
        lib.vs_synth_generate.argtypes = [ctypes.POINTER(SynthConfig), P, P, P]
        sig = {
            "or_depth_to_m": (None, [P, I, F, P]),
            "or_gaussian_table": (None, [F, I, P]),
            "or_bilateral": (None, [P, I, I, P]),
            "or_pyramid_down": (None, [P, I, I, P]),
            "or_point_normal_map": (None, [P, I, I, P, P, P]),
            "or_level_intrinsics": (None, [P, I, P]),
            "or_track": (I, [P, P, P, P, P, P, P, P, P]),
            "or_track_f64": (I, [P, P, P, P, P, P, P, P, P]),
            "or_icp_sums": (I, [P, I, P, P, P, P, P, P]),
            "or_pose_inverse": (None, [P, P]),
            "or_camera_center": (None, [P, P]),
            "or_se3_exp": (None, [P, P]),
            "or_se3_exp_f64": (None, [P, P]),
            "or_volume_create": (P, [P]),
            "or_volume_destroy": (None, [P]),
            "or_volume_reset": (None, [P]),
            "or_volume_get": (None, [P, P, P]),
            "or_volume_set": (None, [P, P, P]),
            "or_volume_flags": (None, [P, P]),
            "or_integrate": (None, [P, P, P, P]),
            "or_raycast": (None, [P, I, P, P, P, P, P, P, P, P]),
            "or_integrate_color": (None, [P, P, P, P, P]),
            "or_volume_get_color": (None, [P, P]),
            "or_volume_set_color": (None, [P, P]),
            "or_raycast_color": (None, [P, I, P, P, P, P, P, P, P, P, P]),
            "or_extract_mesh": (ctypes.c_uint64, [P, P, P, ctypes.c_uint64]),
            "or_render_variant": (None, [P, I, I, P, P, P, P, P, P, P, P, P]),
            "or_update_valid_volume": (ctypes.c_uint32, [P, P]),
            "or_config_geometry": (None, [P, P]),
            "or_prim_cholesky6": (None, [P, P]),
            "or_prim_chol_solve6": (I, [P, P, P]),
            "or_prim_bilinear3": (I, [F, F, I, I, P, I, P]),
            "or_prim_project": (None, [P, P, P]),
            "or_prim_back_project": (None, [F, F, P, F, P]),
            "or_prim_transform": (None, [P, P, I, P]),
            "or_prim_pos_in_voxel": (I, [P, P, P, F, P]),
            "or_prim_pos_in_world": (None, [P, P, F, P]),
            "or_prim_icp_term": (I, [I, I, I, I, P, P, P, P, P, F, P, P]),
            "or_warp_depth": (None, [P, I, I, P, P, P, I, I, P]),
            "or_session_create": (P, [P]),
            "or_session_create_f64": (P, [P]),
            "or_session_destroy": (None, [P]),
            "or_session_frame": (I, [P, P]),
            "or_session_pose": (None, [P, P]),
            "or_session_pose_f64": (None, [P, P]),
            "or_session_volume": (P, [P]),
            "or_session_maps": (None, [P, I, P, P, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def load_ref_pin():
    """The reference's own host math compiled from its source (None when absent)."""
    global _ref
    if _ref is None:
        import build_oracle as _b
        path = _b.build_ref_pin()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        lib.ref_se3_exp.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.ref_inverse4.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.ref_inverse4.restype = ctypes.c_int
        lib.ref_matmul4.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _ref = lib
    return _ref


_ref_cuda = None


def load_ref_pin_cuda():
    """The reference's own device math header compiled as host code (None when absent)."""
    global _ref_cuda
    if _ref_cuda is None:
        import build_oracle as _b
        path = _b.build_ref_pin_cuda()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        sig = {
            "ref_lld6": (I, [P, P]), "ref_sls6": (I, [P, P, P]),
            "ref_giv": (I, [F, F, I, I, P, P]), "ref_gin": (I, [F, F, I, I, P, P]),
            "ref_project": (None, [P, P, P]), "ref_back_project": (None, [F, F, P, F, P]),
            "ref_transform": (None, [P, P, P]), "ref_rotate": (None, [P, P, P]),
            "ref_camera_center": (None, [P, P]),
            "ref_pos_in_voxel": (I, [P, P, P, F, P]), "ref_pos_in_world": (None, [P, P, P, F, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _ref_cuda = lib
    return _ref_cuda


_ref_gpu = None


def load_ref_pin_gpu():
    """The reference's renderer, integrator, tracker and bilateral filter run as
    host code: (render, integ, track, imgproc) libraries, or None when the
    reference tree is absent."""
    global _ref_gpu
    if _ref_gpu is None:
        import build_oracle as _b
        paths = _b.build_ref_pin_gpu()
        if paths is None:
            return None
        r, i, t, b = (ctypes.CDLL(paths[k]) for k in ("render", "integ", "track", "imgproc"))
        P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        r.ref_render_icp.restype = I
        r.ref_render_icp.argtypes = [I, I, P, I, P, P, P, F, F, F, P, P, P, P, P, P, P, P, P, P]
        i.ref_integrate_color.restype = I
        i.ref_integrate_color.argtypes = [I, I, P, P, P, P, F, F, F, P, P, P, P, P, P, P, P]
        r.ref_render_variant.restype = I
        r.ref_render_variant.argtypes = [I, I, I, P, I, P, P, P, F, F, F, P, P, P, P, P, P, P, P, P, P, P, P]
        t.ref_icp_terms.restype = None
        t.ref_icp_terms.argtypes = [I, I, P, P, P, P, P, P, F, P, P, P]
        t.ref_track_pose.restype = I
        t.ref_track_pose.argtypes = [I, I, P, F, P, P, P, P, P, P, P]
        b.ref_bilateral.restype = None
        b.ref_bilateral.argtypes = [I, I, P, P]
        _ref_gpu = (r, i, t, b)
    return _ref_gpu


_ref_cpu = None


def load_ref_pin_cpu():
    """The reference's CPU pyramid, point / normal map and intrinsics
    functions: the library, or None when the reference tree is absent."""
    global _ref_cpu
    if _ref_cpu is None:
        import build_oracle as _b
        path = _b.build_ref_pin_cpu()
        if path is None:
            return None
        lib = ctypes.CDLL(path)
        P, I = ctypes.c_void_p, ctypes.c_int
        lib.ref_depth_pyramid.restype = None
        lib.ref_depth_pyramid.argtypes = [P, I, I, I, P]
        lib.ref_point_normal_map.restype = None
        lib.ref_point_normal_map.argtypes = [P, I, I, P, P, P]
        lib.ref_warp_depth.restype = None
        lib.ref_warp_depth.argtypes = [P, I, I, P, P, P, I, I, P]
        lib.ref_level_intrinsics.restype = None
        lib.ref_level_intrinsics.argtypes = [P, I, P]
        _ref_cpu = lib
    return _ref_cpu


def config_from_vs(vs_cfg, reduce_mode=None, tsdf_store=None):
    """or_config equivalent to a vs_config (field by field)."""
    c = OrConfig()
    for f in ("width", "height", "fx", "fy", "cx", "cy", "levels", "voxel_size", "mu", "max_w", "th_icp",
              "cos_normal", "depth_scale"):
        setattr(c, f, getattr(vs_cfg, f))
    for k in range(3):
        c.dim[k] = vs_cfg.dim[k]
        c.origin[k] = vs_cfg.origin[k]
        c.icp_iters[k] = vs_cfg.icp_iters[k]
    c.reduce_mode = ORACLE_REDUCE_FROM_VS[vs_cfg.reduce_mode] if reduce_mode is None else reduce_mode
    c.tsdf_store = ORACLE_STORE_FROM_VS[vs_cfg.tsdf_type] if tsdf_store is None else tsdf_store
    return c


def make_config(width, height, fx, fy, cx, cy, dim, origin, voxel_size, mu, levels=3, max_w=100.0,
                th_icp=0.01, cos_normal=-3.0, icp_iters=(10, 5, 4), tsdf_store=1, reduce_mode=3,
                depth_scale=0.001):
    c = OrConfig()
    c.width, c.height = width, height
    c.fx, c.fy, c.cx, c.cy = fx, fy, cx, cy
    c.levels = levels
    for k in range(3):
        c.dim[k] = dim[k] if hasattr(dim, "__len__") else dim
        c.origin[k] = origin[k]
        c.icp_iters[k] = icp_iters[k]
    c.voxel_size, c.mu, c.max_w, c.th_icp, c.cos_normal = voxel_size, mu, max_w, th_icp, cos_normal
    c.tsdf_store, c.reduce_mode, c.depth_scale = tsdf_store, reduce_mode, depth_scale
    return c


def level_sizes(cfg):
    w, h = cfg.width, cfg.height
    out = []
    for _ in range(cfg.levels):
        out.append((w, h))
        w //= 2
        h //= 2
    return out


def level_K(cfg):
    K0 = np.array([cfg.fx, cfg.fy, cfg.cx, cfg.cy], np.float32)
    out = np.zeros(12, np.float32)
    load().or_level_intrinsics(_p(K0), 3, _p(out))
    return out.reshape(3, 4)


def warp_depth(depth_m, Kd, T_rgb_wrt_d, Kr, wr, hr):
    """depth seen from the colour camera (z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates)"""
    d = np.ascontiguousarray(depth_m, np.float32)
    hd, wd = d.shape
    out = np.empty((hr, wr), np.float32)
    load().or_warp_depth(_p(d), wd, hd, _p(np.asarray(Kd, np.float32)), _p(np.asarray(T_rgb_wrt_d, np.float32).ravel()),
                         _p(np.asarray(Kr, np.float32)), wr, hr, _p(out))
    return out


class SynthConfig(ctypes.Structure):
    """vs_synth_config (the synthetic-input generator compiled into the
    oracle library, the same source as the package's)"""
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


def synth_config(width, height, **kw):
    lib = load()
    c = SynthConfig()
    lib.vs_synth_default(ctypes.byref(c), width, height)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def synth_generate(cfg):
    """(depth uint16 [n,h,w], T_gc float64 [n,4,4], scene centre) from the
    oracle library's copy of the generator (bit-identical to the package's)"""
    lib = load()
    n, h, w = cfg.n_frames, cfg.height, cfg.width
    depth = np.empty((n, h, w), np.uint16)
    T = np.empty((n, 4, 4), np.float64)
    c = np.empty(3, np.float64)
    if lib.vs_synth_generate(ctypes.byref(cfg), _p(depth), _p(T), _p(c)) != 0:
        raise ValueError("bad synth config")
    return depth, T, c


def depth_to_m(mm, scale=0.001):
    mm = np.ascontiguousarray(mm, np.uint16)
    out = np.empty(mm.shape, np.float32)
    load().or_depth_to_m(_p(mm), mm.size, scale, _p(out))
    return out


def bilateral(depth):
    d = np.ascontiguousarray(depth, np.float32)
    out = np.empty_like(d)
    load().or_bilateral(_p(d), d.shape[1], d.shape[0], _p(out))
    return out


def pyramid_down(depth):
    d = np.ascontiguousarray(depth, np.float32)
    h, w = d.shape
    out = np.empty((h // 2, w // 2), np.float32)
    load().or_pyramid_down(_p(d), w, h, _p(out))
    return out


def point_normal_map(depth, K):
    d = np.ascontiguousarray(depth, np.float32)
    h, w = d.shape
    K = np.ascontiguousarray(K, np.float32)
    v = np.empty((h, w, 3), np.float32)
    n = np.empty((h, w, 3), np.float32)
    load().or_point_normal_map(_p(d), w, h, _p(K), _p(v), _p(n))
    return v, n


def _ptr_array(arrs):
    t = ctypes.c_void_p * 3
    keep = [np.ascontiguousarray(a, np.float32) if a is not None else None for a in arrs]
    ptrs = t(*[(a.ctypes.data if a is not None else None) for a in keep] + [None] * (3 - len(keep)))
    return ptrs, keep


def track(cfg, depth_levels, mvtx_levels, mnrm_levels, T_gc_prev, innrm_levels=None, init_T12=None, f64=False):
    """Returns (ok, T_gc_out [4x4], info[2])."""
    dp, k1 = _ptr_array(depth_levels)
    vp, k2 = _ptr_array(mvtx_levels)
    np_, k3 = _ptr_array(mnrm_levels)
    ip = None
    if innrm_levels is not None:
        ip, k4 = _ptr_array(innrm_levels)
    info = np.zeros(2, np.int32)
    lib = load()
    if f64:
        Tp = np.ascontiguousarray(T_gc_prev, np.float64).reshape(16)
        init = None if init_T12 is None else np.ascontiguousarray(init_T12, np.float64).reshape(16)
        out = np.empty(16, np.float64)
        ok = lib.or_track_f64(ctypes.byref(cfg), dp, vp, np_, ip, _p(Tp), _p(init), _p(out), _p(info))
    else:
        Tp = np.ascontiguousarray(T_gc_prev, np.float32).reshape(16)
        init = None if init_T12 is None else np.ascontiguousarray(init_T12, np.float32).reshape(16)
        out = np.empty(16, np.float32)
        ok = lib.or_track(ctypes.byref(cfg), dp, vp, np_, ip, _p(Tp), _p(init), _p(out), _p(info))
    return bool(ok), out.reshape(4, 4), info


def icp_sums(cfg, level, depth, mvtx, mnrm, T21, innrm=None):
    out = np.zeros(29, np.float64)
    d = np.ascontiguousarray(depth, np.float32)
    v = np.ascontiguousarray(mvtx, np.float32)
    n = np.ascontiguousarray(mnrm, np.float32)
    i = None if innrm is None else np.ascontiguousarray(innrm, np.float32)
    T = np.ascontiguousarray(T21, np.float32).reshape(16)
    load().or_icp_sums(ctypes.byref(cfg), level, _p(d), _p(v), _p(n), _p(i), _p(T), _p(out))
    return out


def pose_inverse(T):
    T = np.ascontiguousarray(T, np.float32).reshape(16)
    out = np.empty(16, np.float32)
    load().or_pose_inverse(_p(T), _p(out))
    return out.reshape(4, 4)


def camera_center(T_gc):
    T = np.ascontiguousarray(T_gc, np.float32).reshape(16)
    out = np.empty(3, np.float32)
    load().or_camera_center(_p(T), _p(out))
    return out


def se3_exp(xi, f64=False):
    if f64:
        x = np.ascontiguousarray(xi, np.float64)
        out = np.empty(16, np.float64)
        load().or_se3_exp_f64(_p(x), _p(out))
    else:
        x = np.ascontiguousarray(xi, np.float32)
        out = np.empty(16, np.float32)
        load().or_se3_exp(_p(x), _p(out))
    return out.reshape(4, 4)


class Volume:
    def __init__(self, cfg, handle=None, owner=True):
        self.lib = load()
        self.cfg = cfg
        self.h = handle if handle is not None else self.lib.or_volume_create(ctypes.byref(cfg))
        self.owner = owner
        self.n = cfg.dim[0] * cfg.dim[1] * cfg.dim[2]

    def __del__(self):
        if self.owner and self.h:
            self.lib.or_volume_destroy(self.h)
            self.h = None

    def get(self):
        t = np.empty(self.n, np.float32)
        w = np.empty(self.n, np.uint16)
        self.lib.or_volume_get(self.h, _p(t), _p(w))
        return t, w

    def set(self, tsdf, weight):
        t = np.ascontiguousarray(tsdf, np.float32)
        w = np.ascontiguousarray(weight, np.uint16)
        self.lib.or_volume_set(self.h, _p(t), _p(w))

    def flags(self):
        nb = (self.cfg.dim[0] // 8) * (self.cfg.dim[1] // 8) * (self.cfg.dim[2] // 8)
        f = np.empty(nb, np.uint8)
        self.lib.or_volume_flags(self.h, _p(f))
        return f

    def integrate(self, depth_m, T_gc, T_cg):
        d = np.ascontiguousarray(depth_m, np.float32)
        a = np.ascontiguousarray(T_gc, np.float32).reshape(16)
        b = np.ascontiguousarray(T_cg, np.float32).reshape(16)
        self.lib.or_integrate(self.h, _p(d), _p(a), _p(b))

    def integrate_color(self, depth_m, rgb, T_gc, T_cg):
        """rgb: planar uint8 (3, h, w) of the depth image's size"""
        d = np.ascontiguousarray(depth_m, np.float32)
        c = np.ascontiguousarray(rgb, np.uint8)
        a = np.ascontiguousarray(T_gc, np.float32).reshape(16)
        b = np.ascontiguousarray(T_cg, np.float32).reshape(16)
        self.lib.or_integrate_color(self.h, _p(d), _p(c), _p(a), _p(b))

    def get_color(self):
        out = np.empty(3 * self.n, np.uint8)
        self.lib.or_volume_get_color(self.h, _p(out))
        return out.reshape(3, self.n)

    def set_color(self, rgb):
        c = np.ascontiguousarray(rgb, np.uint8)
        assert c.size == 3 * self.n
        self.lib.or_volume_set_color(self.h, _p(c))

    def mesh(self, with_color=False):
        n = self.lib.or_extract_mesh(self.h, None, None, 0)
        xyz = np.empty((max(n, 1), 3, 3), np.float32)
        rgb = np.empty((max(n, 1), 3, 3), np.uint8) if with_color else None
        self.lib.or_extract_mesh(self.h, _p(xyz), _p(rgb) if with_color else None, n)
        return xyz[:n], (rgb[:n] if with_color else None)

    def raycast_color(self, level, T_gc, T_cg, cam, light=(0.0, 0.0, -1.0)):
        w, h = level_sizes(self.cfg)[level]
        a = np.ascontiguousarray(T_gc, np.float32).reshape(16)
        b = np.ascontiguousarray(T_cg, np.float32).reshape(16)
        c = np.ascontiguousarray(cam, np.float32)
        l = np.ascontiguousarray(light, np.float32)
        dep = np.empty((h, w), np.float32)
        v = np.empty((h, w, 3), np.float32)
        n = np.empty((h, w, 3), np.float32)
        img = np.empty((h, w), np.uint8)
        rgb = np.empty((3, h, w), np.uint8)
        self.lib.or_raycast_color(self.h, level, _p(a), _p(b), _p(c), _p(l), _p(dep), _p(v), _p(n), _p(img),
                                  _p(rgb))
        return dep, v, n, img, rgb

    def render_variant(self, mode, level, T_gc, T_cg, cam, light=(0.0, 0.0, -1.0), vertex=True, color=False):
        """mode: RAY_* bits; returns depth, vertex (or None), normals, image, colour (or None)"""
        w, h = level_sizes(self.cfg)[level]
        a = np.ascontiguousarray(T_gc, np.float32).reshape(16)
        b = np.ascontiguousarray(T_cg, np.float32).reshape(16)
        c = np.ascontiguousarray(cam, np.float32)
        l = np.ascontiguousarray(light, np.float32)
        dep = np.empty((h, w), np.float32)
        v = np.empty((h, w, 3), np.float32) if vertex else None
        n = np.empty((h, w, 3), np.float32)
        img = np.empty((h, w), np.uint8)
        rgb = np.empty((3, h, w), np.uint8) if color else None
        self.lib.or_render_variant(self.h, level, mode, _p(a), _p(b), _p(c), _p(l), _p(dep), _p(v) if vertex else None,
                                   _p(n), _p(img), _p(rgb) if color else None)
        return dep, v, n, img, rgb

    def update_valid_volume(self, valid):
        """valid: one byte per voxel, x fastest; returns the sub-cubes reset"""
        m = np.ascontiguousarray(valid, np.uint8).reshape(-1)
        assert m.size == self.n
        return int(self.lib.or_update_valid_volume(self.h, _p(m)))

    def raycast(self, level, T_gc, T_cg, cam, light=(0.0, 0.0, -1.0)):
        w, h = level_sizes(self.cfg)[level]
        a = np.ascontiguousarray(T_gc, np.float32).reshape(16)
        b = np.ascontiguousarray(T_cg, np.float32).reshape(16)
        c = np.ascontiguousarray(cam, np.float32)
        l = np.ascontiguousarray(light, np.float32)
        dep = np.empty((h, w), np.float32)
        v = np.empty((h, w, 3), np.float32)
        n = np.empty((h, w, 3), np.float32)
        img = np.empty((h, w), np.uint8)
        self.lib.or_raycast(self.h, level, _p(a), _p(b), _p(c), _p(l), _p(dep), _p(v), _p(n), _p(img))
        return dep, v, n, img


class Session:
    def __init__(self, cfg, f64=False):
        self.lib = load()
        self.cfg = cfg
        self.f64 = f64
        self.h = (self.lib.or_session_create_f64 if f64 else self.lib.or_session_create)(ctypes.byref(cfg))

    def __del__(self):
        if self.h:
            self.lib.or_session_destroy(self.h)
            self.h = None

    def frame(self, depth_mm):
        d = np.ascontiguousarray(depth_mm, np.uint16)
        return bool(self.lib.or_session_frame(self.h, _p(d)))

    def pose(self):
        out = np.empty(16, np.float32)
        self.lib.or_session_pose(self.h, _p(out))
        return out.reshape(4, 4)

    def pose_f64(self):
        out = np.empty(16, np.float64)
        self.lib.or_session_pose_f64(self.h, _p(out))
        return out.reshape(4, 4)

    def volume(self):
        return Volume(self.cfg, handle=self.lib.or_session_volume(self.h), owner=False)

    def maps(self, level):
        w, h = level_sizes(self.cfg)[level]
        md = np.empty((h, w), np.float32)
        mv = np.empty((h, w, 3), np.float32)
        mn = np.empty((h, w, 3), np.float32)
        idp = np.empty((h, w), np.float32)
        self.lib.or_session_maps(self.h, level, _p(md), _p(mv), _p(mn), _p(idp))
        return dict(model_depth=md, model_vertex=mv, model_normal=mn, input_depth=idp)

"""Regenerates the committed golden fixtures (run from the repository root,
in a checkout that has the reference tree mounted; TEST INFRASTRUCTURE ONLY).

refpin.npz
    SE(3) exponentials and 4x4 inverses computed by the reference's own
    STAC/Util/_yooji_math_inlines.h (d_cme_Compute_Matrix_Exponential,
    d_im_Inverse_Matrix_4x4, d_mmm_Multiply_Matrix_Matrix), compiled from the
    reference tree by oracle/build_oracle.py.  These pin the oracle's pose
    algebra bit for bit.
refpin_cuda.npz
    Inputs and outputs of the reference's own STAC/Util/_yooji_cuda_math.h
    helpers, compiled as host C++ (oracle/ref_pin_cuda.cpp with the stand-ins
    of oracle/ref_shim/): 6x6 Cholesky factors and solves
    (d_lld_LL_Decomposition, d_sls_Solve_Linear_System_using_LLD, including
    singular and negative-pivot systems), bilinear vertex / normal lookups
    (d_giv / d_gin, with -100 sentinels and integer coordinates), projection,
    back-projection, transform, rotation, camera centre and voxel / world
    positions.  These pin the oracle's restatements of them bit for bit.
refpin_gpu.npz
    Two frames (80x60 depth with a zero border and a colour image with no zero
    texel, so every colour sample interpolates) integrated into a 48^3 cube,
    and the ray-cast maps of every pyramid level from a third pose, computed
    by the reference's own renderer and integrator sources run as host code
    (oracle/ref_pin_gpu.cpp): float TSDF, uchar weights and colour after each
    frame, depth / vertex / normal / shading per level.  These pin the
    oracle's integration and ray-cast bit for bit.
seq_small.npz
    A 6-frame 160x120 synthetic sequence (uint16 input frames stored, so no
    cross-host generator identity is assumed) and the oracle's outputs for it
    (96^3 int16 volume over 0.75 m): per-frame poses and tracking flags, final
    weights / quantised TSDF, and the level-0 model depth of the last frame.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "vcl-volume-scanner_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_py as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def refpin():
    ref = O.load_ref_pin()
    if ref is None:
        raise SystemExit("the reference tree is not mounted; refpin.npz cannot be regenerated")
    rng = np.random.default_rng(20240601)
    n = 64
    mags = np.concatenate([np.full(16, 1e-4), np.full(16, 1e-3), np.full(16, 1e-2), np.full(16, 1e-1)])
    xi = (rng.standard_normal((n, 6)) * mags[:, None]).astype(np.float32)
    exp = np.empty((n, 16), np.float32)
    for i in range(n):
        ref.ref_se3_exp(xi[i].ctypes.data_as(ctypes.c_void_p), exp[i].ctypes.data_as(ctypes.c_void_p))
    # rigid matrices from products of exponentials, then the reference inverse
    mats = np.empty((n, 16), np.float32)
    inv = np.empty((n, 16), np.float32)
    for i in range(n):
        a = exp[i].copy()
        b = exp[(i * 7 + 3) % n].copy()
        ref.ref_matmul4(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                        mats[i].ctypes.data_as(ctypes.c_void_p))
        mats[i, 3] += np.float32(0.3 * np.sin(i))
        mats[i, 7] += np.float32(-0.2 * np.cos(i))
        mats[i, 11] += np.float32(1.0 + 0.1 * i / n)
        ref.ref_inverse4(mats[i].ctypes.data_as(ctypes.c_void_p), inv[i].ctypes.data_as(ctypes.c_void_p))
    np.savez_compressed(os.path.join(OUT, "refpin.npz"), xi=xi, exp=exp, mats=mats, inv=inv)


def seq_small():
    import helpers
    case = helpers.make_case(width=160, height=120, dim=96, frames=6, seed=11, size=0.75)
    depth, ocfg = case["depth"], case["ocfg"]
    s = O.Session(ocfg)
    poses = []
    tracked = []
    for k in range(depth.shape[0]):
        tracked.append(s.frame(depth[k]))
        poses.append(s.pose())
    assert all(tracked)
    t, w = s.volume().get()
    m = s.maps(0)
    c = case["cfg"]
    cfg_arr = np.array([c.width, c.height, c.fx, c.fy, c.cx, c.cy, c.dim[0], c.origin[0], c.origin[1], c.origin[2],
                        c.voxel_size, c.mu, c.th_icp], np.float64)
    np.savez_compressed(os.path.join(OUT, "seq_small.npz"), depth=depth, poses=np.array(poses),
                        tracked=np.array(tracked), weight=w,
                        tsdf_q=helpers.q16(t).astype(np.int16), model_depth=m["model_depth"], cfg=cfg_arr,
                        gt=case["gt"])


def refpin_cuda():
    ref = O.load_ref_pin_cuda()
    if ref is None:
        raise SystemExit("the reference tree is not mounted; refpin_cuda.npz cannot be regenerated")
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rng = np.random.default_rng(20240602)
    # 6x6 systems: well and badly conditioned, singular, a negative pivot
    n = 48
    A = np.empty((n, 36), np.float32)
    for i in range(n):
        M = rng.standard_normal((6, 6)).astype(np.float32) * np.float32(10.0 ** (i % 7 - 3))
        a = (M @ M.T).astype(np.float32)
        if i % 8 == 6:
            a[3, :] = 0.0
            a[:, 3] = 0.0
        if i % 8 == 7:
            a[2, 2] = -1.0
        A[i] = a.reshape(36)
    rhs = rng.standard_normal((n, 6)).astype(np.float32)
    L = np.zeros((n, 36), np.float32)
    x = np.zeros((n, 6), np.float32)
    ok = np.zeros(n, np.int32)
    for i in range(n):
        ref.ref_lld6(p(A[i]), p(L[i]))
        ok[i] = ref.ref_sls6(p(L[i]), p(rhs[i]), p(x[i]))
    # bilinear lookups on one 13x9 map with sentinels
    w, h = 13, 9
    mp = rng.standard_normal((h, w, 3)).astype(np.float32)
    mp[rng.random((h, w)) < 0.12] = -100.0
    mp = np.ascontiguousarray(mp.reshape(-1))
    m = 400
    xy = np.stack([rng.uniform(-0.5, w - 0.5, m), rng.uniform(-0.5, h - 0.5, m)], 1).astype(np.float32)
    xy[::4, 0] = np.floor(xy[::4, 0])
    xy[1::4, 1] = np.floor(xy[1::4, 1])
    giv = np.zeros((m, 3), np.float32)
    gin = np.zeros((m, 3), np.float32)
    giv_ok = np.zeros(m, np.int32)
    gin_ok = np.zeros(m, np.int32)
    for i in range(m):
        giv_ok[i] = ref.ref_giv(float(xy[i, 0]), float(xy[i, 1]), w, h, p(mp), p(giv[i]))
        gin_ok[i] = ref.ref_gin(float(xy[i, 0]), float(xy[i, 1]), w, h, p(mp), p(gin[i]))
    # geometry
    g = 200
    K = np.stack([rng.uniform(100, 600, g), rng.uniform(100, 600, g), rng.uniform(100, 400, g),
                  rng.uniform(80, 300, g)], 1).astype(np.float32)
    p3 = (rng.standard_normal((g, 3)) * [0.5, 0.5, 0.3] + [0, 0, 1.2]).astype(np.float32)
    T = rng.standard_normal((g, 16)).astype(np.float32)
    uvd = np.stack([rng.uniform(0, 640, g), rng.uniform(0, 480, g), rng.uniform(0.3, 3, g)], 1).astype(np.float32)
    org = rng.uniform(-1, 0, (g, 3)).astype(np.float32)
    dim = np.array([128, 96, 64], np.int32)
    inv = rng.uniform(50, 500, g).astype(np.float32)
    q = (org + rng.uniform(-0.1, 1.2, (g, 3))).astype(np.float32)
    vox = rng.uniform(-1, 130, (g, 3)).astype(np.float32)
    proj = np.zeros((g, 2), np.float32)
    bproj = np.zeros((g, 3), np.float32)
    trans = np.zeros((g, 3), np.float32)
    rot = np.zeros((g, 3), np.float32)
    cen = np.zeros((g, 3), np.float32)
    gpv = np.zeros((g, 3), np.float32)
    gpv_ok = np.zeros(g, np.int32)
    gpw = np.zeros((g, 3), np.float32)
    for i in range(g):
        ref.ref_project(p(p3[i]), p(K[i]), p(proj[i]))
        ref.ref_back_project(float(uvd[i, 0]), float(uvd[i, 1]), p(K[i]), float(uvd[i, 2]), p(bproj[i]))
        ref.ref_transform(p(p3[i]), p(T[i]), p(trans[i]))
        ref.ref_rotate(p(p3[i]), p(T[i]), p(rot[i]))
        ref.ref_camera_center(p(T[i]), p(cen[i]))
        gpv_ok[i] = ref.ref_pos_in_voxel(p(q[i]), p(org[i]), p(dim), float(inv[i]), p(gpv[i]))
        ref.ref_pos_in_world(p(vox[i]), p(org[i]), p(dim), float(inv[i]), p(gpw[i]))
    np.savez_compressed(os.path.join(OUT, "refpin_cuda.npz"), A=A, rhs=rhs, L=L, x=x, ok=ok, w=w, h=h, map=mp, xy=xy,
                        giv=giv, gin=gin, giv_ok=giv_ok, gin_ok=gin_ok, K=K, p3=p3, T=T, uvd=uvd, org=org, dim=dim,
                        inv=inv, q=q, vox=vox, proj=proj, bproj=bproj, trans=trans, rot=rot, cen=cen, gpv=gpv,
                        gpv_ok=gpv_ok, gpw=gpw)


def refpin_gpu():
    libs = O.load_ref_pin_gpu()
    if libs is None:
        raise SystemExit("the reference tree is not mounted; refpin_gpu.npz cannot be regenerated")
    rr, ri, rt, rb = libs
    import vs_scanner as V
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    w, h, dim, size = 80, 60, 48, 0.75
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=3, seed=9, dropout_iid=0.01)
    depth_mm, rgb, gt, centre = V.synth_generate_rgb(sc)
    origin, vox = V.cube_around(centre, size, dim)
    cfg = dict(width=w, height=h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=dim, origin=np.array(origin, np.float32),
               voxel_size=vox, mu=0.03, max_w=100.0)
    oc = refpin_gpu_config(cfg)
    geo = np.zeros(5, np.float32)
    O.load().or_config_geometry(ctypes.byref(oc), p(geo))
    K0 = np.array([oc.fx, oc.fy, oc.cx, oc.cy], np.float32)
    dims = np.array([dim] * 3, np.int32)
    org = np.array(list(oc.origin), np.float32)
    cen = np.ascontiguousarray(geo[:3])
    n = dim ** 3
    t = np.ones(n, np.float32)
    wt = np.zeros(n, np.uint8)
    col = np.zeros(3 * n, np.uint8)
    depths, imgs, tsdf, weight, colour = [], [], [], [], []
    for k in range(2):
        raw = O.depth_to_m(depth_mm[k]).astype(np.float32)
        raw[0, :] = raw[-1, :] = raw[:, 0] = raw[:, -1] = 0.0
        img = np.ascontiguousarray(np.maximum(rgb[k], 1), np.uint8)
        Tgc = np.ascontiguousarray(gt[k], np.float32)
        Tcg = O.pose_inverse(Tgc)
        ri.ref_integrate_color(w, h, p(K0), p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(t), p(wt),
                               p(col), p(np.ascontiguousarray(raw)), p(img), p(Tgc), p(np.ascontiguousarray(Tcg)), None)
        depths.append(raw)
        imgs.append(img)
        tsdf.append(t.copy())
        weight.append(wt.copy())
        colour.append(col.copy())
    Tgc = np.ascontiguousarray(gt[2], np.float32)
    Tcg = np.ascontiguousarray(O.pose_inverse(Tgc))
    cam = np.ascontiguousarray(O.camera_center(Tgc), np.float32)
    light = np.array([0, 0, -1], np.float32)
    maps = {}
    for l in range(3):
        lw, lh = w >> l, h >> l
        d, v, nn, im = (np.zeros(lw * lh, np.float32), np.zeros(3 * lw * lh, np.float32),
                        np.zeros(3 * lw * lh, np.float32), np.zeros(lw * lh, np.uint8))
        rr.ref_render_icp(w, h, p(K0), l, p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(t), p(wt),
                          p(Tgc), p(Tcg), p(cam), p(light), p(d), p(v), p(nn), p(im))
        maps.update({"depth%d" % l: d, "vertex%d" % l: v, "normal%d" % l: nn, "img%d" % l: im})
    # the per-pixel ICP term against the level-1 model maps: the next frame's
    # depth, subsampled, and an increment a little off the identity
    icp = icp_case(np.ascontiguousarray(O.depth_to_m(depth_mm[2])[::2, ::2], np.float32))
    K1 = np.array([oc.fx / 2, oc.fy / 2, oc.cx / 2, oc.cy / 2], np.float32)
    n1 = (w >> 1) * (h >> 1)
    ATA, ATb, ok = np.zeros((n1, 36), np.float32), np.zeros((n1, 6), np.float32), np.zeros(n1, np.uint8)
    rt.ref_icp_terms(w >> 1, h >> 1, p(K1), p(icp["depth"]), p(maps["depth1"]), p(maps["vertex1"]), p(maps["normal1"]),
                     p(icp["T21"]), 0.01, p(ATA), p(ATb), p(ok))
    maps.update({"icp_depth": icp["depth"], "icp_T21": icp["T21"], "icp_K": K1, "icp_ATA": ATA, "icp_ATb": ATb,
                 "icp_ok": ok})
    # the scene renders of the colour cube at pose 2
    for var, (mode, level, has_v) in RENDER_VARIANTS.items():
        lw, lh = w >> level, h >> level
        d, v, nn, im, ci = (np.zeros(lw * lh, np.float32), np.zeros(3 * lw * lh, np.float32),
                            np.zeros(3 * lw * lh, np.float32), np.zeros(lw * lh, np.uint8),
                            np.zeros(3 * lw * lh, np.uint8))
        rr.ref_render_variant(var, w, h, p(K0), level, p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(t),
                              p(wt), p(col), p(Tgc), p(Tcg), p(cam), p(light), p(d), p(v), p(nn), p(im), p(ci))
        maps.update({"var%d_depth" % var: d, "var%d_normal" % var: nn, "var%d_img" % var: im, "var%d_rgb" % var: ci})
        if has_v:
            maps["var%d_vertex" % var] = v
    # a third integration (frame 2) followed by carving with carve_mask
    raw = O.depth_to_m(depth_mm[2]).astype(np.float32)
    raw[0, :] = raw[-1, :] = raw[:, 0] = raw[:, -1] = 0.0
    img = np.ascontiguousarray(np.maximum(rgb[2], 1), np.uint8)
    mask = carve_mask(dim)
    ri.ref_integrate_color(w, h, p(K0), p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(t), p(wt), p(col),
                           p(np.ascontiguousarray(raw)), p(img), p(Tgc), p(Tcg), p(mask))
    maps.update({"carve_depth": raw, "carve_rgb": img, "carve_tsdf": t.copy(), "carve_weight": wt.copy(),
                 "carve_colour": col.copy()})
    # the bilateral filter of the raw frame with holes of each kind
    bil = bilateral_input(O.depth_to_m(depth_mm[0]))
    out = np.zeros_like(bil)
    rb.ref_bilateral(w, h, p(bil), p(out))
    maps.update({"bil_in": bil, "bil_out": out})
    np.savez_compressed(os.path.join(OUT, "refpin_gpu.npz"), cfg_w=w, cfg_h=h, cfg_f=f, cfg_dim=dim,
                        cfg_origin=cfg["origin"], cfg_vox=vox, cfg_mu=0.03, cfg_maxw=100.0, depth=np.stack(depths),
                        rgb=np.stack(imgs), T=np.ascontiguousarray(gt[:3], np.float32), tsdf=np.stack(tsdf),
                        weight=np.stack(weight), colour=np.stack(colour), **maps)


# the reference's other renders, by the index of ref_render_variant: the
# oracle's mode bits (scene ray-cast 1, global normals 2, nearest-voxel colour
# 4, white background 8), the pyramid level, and whether a vertex map is made
RENDER_VARIANTS = {0: (1 | 2 | 4, 0, True), 1: (1 | 2, 0, False), 2: (2 | 8, 1, False)}


def carve_mask(dim):
    """valid voxels (one byte each, x fastest) of a slanted half-space
    x + 2 y < 1.2 dim: sub-cubes past it are wholly invalid, those on it mixed"""
    z, y, x = np.meshgrid(np.arange(dim), np.arange(dim), np.arange(dim), indexing="ij")
    return np.ascontiguousarray((x + 2 * y < 1.2 * dim).reshape(-1).astype(np.uint8))


def bilateral_input(depth):
    """a depth frame (metres) with a 30 cm step, single zero texels and zero
    lines one texel wide (averaged into the taps), and 2x2 zero blocks and
    zero lines two texels wide (each makes a hole), one in a corner"""
    d = np.array(depth, np.float32)
    h, w = d.shape
    d[:, (2 * w) // 3:] += 0.3
    d[7, 9] = d[30, 41] = 0.0
    d[h // 3, :] = 0.0
    d[:, w // 4] = 0.0
    d[20:22, 20:22] = 0.0
    d[h - 2:h, w - 2:w] = 0.0
    d[h // 2:h // 2 + 2, :] = 0.0
    d[:, w // 2:w // 2 + 2] = 0.0
    return np.ascontiguousarray(d)


def icp_case(depth):
    """a depth frame and an increment T21 (4x4 row-major float32): a rotation
    of 0.6 degrees about (1, 2, 3) / |.| and a 4 mm shift"""
    a = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    th = np.deg2rad(0.6)
    Kx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    R = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = [0.004, -0.002, 0.003]
    return {"depth": np.ascontiguousarray(depth, np.float32), "T21": np.ascontiguousarray(T, np.float32)}


def track_case(w, h, dim=128, size=0.75, seed=7):
    """the tracking case of refpin_track: frames 0 and 1 integrated at their
    true poses into a float cube, model maps ray-cast at pose 1, frame 2
    filtered into the input pyramid (all by the oracle, whose integration,
    ray-cast and bilateral filter equal the reference's bit for bit).
    Returns (or_config with the reference's tracker settings, raw frames in
    mm, true poses, input depth levels, model depth / vertex / normal levels)."""
    import vs_scanner as V
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=3, seed=seed, dropout_iid=0.01)
    dmm, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, size, dim)
    oc = refpin_gpu_config(dict(width=w, height=h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=dim,
                                origin=np.array(origin, np.float32), voxel_size=vox, mu=0.03, max_w=100.0))
    # the reference's tracker: block-tree reduction, iterations {10, 7, 7},
    # distance threshold (0.055 size)^2
    oc.reduce_mode = 0
    oc.th_icp = float(np.float32((0.055 * size) ** 2))
    for k, n in enumerate((10, 7, 7)):
        oc.icp_iters[k] = n
    vol = O.Volume(oc)
    for k in range(2):
        T = np.ascontiguousarray(gt[k], np.float32)
        vol.integrate(O.depth_to_m(dmm[k]), T, O.pose_inverse(T))
    T1 = np.ascontiguousarray(gt[1], np.float32)
    md, mv, mn = [], [], []
    for l in range(3):
        d, v, n, _ = vol.raycast(l, T1, O.pose_inverse(T1), O.camera_center(T1))
        md.append(np.ascontiguousarray(d))
        mv.append(np.ascontiguousarray(v))
        mn.append(np.ascontiguousarray(n))
    ind = [np.ascontiguousarray(O.bilateral(O.depth_to_m(dmm[2])), np.float32)]
    for l in range(2):
        ind.append(np.ascontiguousarray(O.pyramid_down(ind[-1]), np.float32))
    return oc, dmm, np.ascontiguousarray(gt, np.float32), ind, md, mv, mn


def ref_track(rt, oc, ind, md, mv, mn, T_prev, init):
    """the reference's tp_Track_Pose on these inputs: (ok, T_gc out)"""
    pa = lambda arrs: (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    K0 = np.array([oc.fx, oc.fy, oc.cx, oc.cy], np.float32)
    out = np.zeros(16, np.float32)
    init_p = None if init is None else np.ascontiguousarray(init, np.float32).ctypes.data_as(ctypes.c_void_p)
    ok = rt.ref_track_pose(oc.width, oc.height, K0.ctypes.data_as(ctypes.c_void_p), oc.th_icp, pa(ind), pa(md),
                           pa(mv), pa(mn), np.ascontiguousarray(T_prev, np.float32).ctypes.data_as(ctypes.c_void_p),
                           init_p, out.ctypes.data_as(ctypes.c_void_p))
    return ok, out.reshape(4, 4)


def refpin_track():
    """the reference's whole tp_Track_Pose (160x120, three levels; and level 0
    only from an identity initial increment), its block trees run as
    cooperative threads; about a minute"""
    libs = O.load_ref_pin_gpu()
    if libs is None:
        raise SystemExit("the reference tree is not mounted; refpin_track.npz cannot be regenerated")
    w, h = 160, 120
    oc, dmm, gt, ind, md, mv, mn = track_case(w, h)
    ok0, T0 = ref_track(libs[2], oc, ind, md, mv, mn, gt[1], None)
    ok1, T1 = ref_track(libs[2], oc, ind, md, mv, mn, gt[1], np.eye(4, dtype=np.float32))
    np.savez_compressed(os.path.join(OUT, "refpin_track.npz"), w=w, h=h, depth_mm=dmm, gt=gt, ok_levels=ok0,
                        T_levels=T0, ok_init=ok1, T_init=T1)


def cpu_case(w, h, seed):
    """a bilateral-filtered depth frame (metres) with holes, zero lines and a
    step, and level-0 intrinsics"""
    import vs_scanner as V
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=1, seed=seed, dropout_iid=0.02)
    d = V.synth_generate(sc)[0]
    x = np.ascontiguousarray(O.bilateral(bilateral_input(O.depth_to_m(d[0]))), np.float32)
    return x, np.array([f, f, w / 2.0, h / 2.0], np.float32)


def ref_cpu_maps(lib, depth, K0, levels=3):
    """the reference's depth pyramid, level intrinsics, and point / normal
    maps of each level: (levels, K (levels x 4), vertices, normals)"""
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    h, w = depth.shape
    sizes = [(w >> l, h >> l) for l in range(levels)]
    flat = np.zeros(sum(a * b for a, b in sizes), np.float32)
    lib.ref_depth_pyramid(p(depth), w, h, levels, p(flat))
    Kl = np.zeros(4 * levels, np.float32)
    lib.ref_level_intrinsics(p(K0), levels, p(Kl))
    lv, vtx, nrm, off = [], [], [], 0
    for l, (a, b) in enumerate(sizes):
        lv.append(flat[off:off + a * b].reshape(b, a).copy())
        off += a * b
        v, n = np.zeros((b, a, 3), np.float32), np.zeros((b, a, 3), np.float32)
        lib.ref_point_normal_map(p(lv[-1]), a, b, p(np.ascontiguousarray(Kl[4 * l:4 * l + 4])), p(v), p(n))
        vtx.append(v)
        nrm.append(n)
    return lv, Kl.reshape(levels, 4), vtx, nrm


def refpin_cpu():
    """the reference's CPU image functions on a 90x66 frame (odd level sizes)"""
    lib = O.load_ref_pin_cpu()
    if lib is None:
        raise SystemExit("the reference tree is not mounted; refpin_cpu.npz cannot be regenerated")
    x, K0 = cpu_case(90, 66, seed=11)
    lv, Kl, vtx, nrm = ref_cpu_maps(lib, x, K0)
    out = {"depth0": x, "K0": K0, "K": Kl}
    for l in range(3):
        out.update({"pyr%d" % l: lv[l], "vertex%d" % l: vtx[l], "normal%d" % l: nrm[l]})
    # the same frame seen from a colour camera beside it (z_tdrcc)
    T, Kr = warp_rig(90, 66)
    warped = np.zeros((66, 90), np.float32)
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)
    lib.ref_warp_depth(p(x), 90, 66, p(K0), p(T), p(Kr), 90, 66, p(warped))
    out.update({"warp_T": T, "warp_Kr": Kr, "warp": warped})
    np.savez_compressed(os.path.join(OUT, "refpin_cpu.npz"), **out)


def warp_rig(w, h):
    """a colour camera 5 cm to the side, turned 3 degrees about y, with its
    own intrinsics: (T depth -> colour 4x4, colour intrinsics)"""
    a = np.deg2rad(3.0)
    T = np.eye(4, dtype=np.float32)
    T[0, 0] = T[2, 2] = np.cos(a)
    T[0, 2], T[2, 0] = np.sin(a), -np.sin(a)
    T[0, 3] = -0.05
    f = 300.0 * w / 320.0
    return T, np.array([f, 0.993 * f, w / 2.0 + 3.5, h / 2.0 - 1.75], np.float32)


def pipeline_case(w=120, h=90, dim=96, size=0.75, frames=4, seed=7):
    """a depth sequence and the or_config of the reference's settings for the
    whole per-frame path (float TSDF, block-tree reduction, ICP {10, 7, 7},
    distance (0.055 size)^2, no normal test)"""
    import vs_scanner as V
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=frames, seed=seed, dropout_iid=0.01)
    dmm, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, size, dim)
    oc = refpin_gpu_config(dict(width=w, height=h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=dim,
                                origin=np.array(origin, np.float32), voxel_size=vox, mu=0.03, max_w=100.0))
    oc.reduce_mode = 0
    oc.th_icp = float(np.float32((0.055 * size) ** 2))
    for k, n in enumerate((10, 7, 7)):
        oc.icp_iters[k] = n
    return oc, dmm


def ref_pipeline(oc, dmm):
    """the per-frame path chained from the reference's own stages, in the
    order of its scanner loop (z_yooji_object_scanner.cpp: z_uid bilateral,
    z_cip pyramid, z_ecp track from the second frame, z_uom integrate the raw
    depth, z_uts ray-cast every level): bilateral (d_bilateral_filter),
    pyramid (cpdd), tp_Track_Pose, cdtocc, rmi_Render_Maps_for_ICP, with the
    reference's inverse (d_im_Inverse_Matrix_4x4) and camera centre (d_gcc).
    Returns (per-frame poses, tracked flags, tsdf, weights, model depth /
    vertex / normal of each level after the last frame)."""
    rr, ri, rt, rb = O.load_ref_pin_gpu()
    cpu, m4, cu = O.load_ref_pin_cpu(), O.load_ref_pin(), O.load_ref_pin_cuda()
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)
    w, h, dim = oc.width, oc.height, oc.dim[0]
    geo = np.zeros(5, np.float32)
    O.load().or_config_geometry(ctypes.byref(oc), p(geo))
    K0 = np.array([oc.fx, oc.fy, oc.cx, oc.cy], np.float32)
    dims, org, cen = np.array([dim] * 3, np.int32), np.array(list(oc.origin), np.float32), np.ascontiguousarray(geo[:3])
    n = dim ** 3
    tsdf, wt, col = np.ones(n, np.float32), np.zeros(n, np.uint8), np.zeros(3 * n, np.uint8)
    rgb = np.full((3, h, w), 128, np.uint8)
    sizes = [(w >> l, h >> l) for l in range(3)]
    T = np.eye(4, dtype=np.float32)
    md = [np.zeros(a * b, np.float32) for a, b in sizes]
    mv = [np.zeros(3 * a * b, np.float32) for a, b in sizes]
    mn = [np.zeros(3 * a * b, np.float32) for a, b in sizes]
    poses, tracked = [], []
    for k in range(dmm.shape[0]):
        raw = np.ascontiguousarray(dmm[k].astype(np.float32) * np.float32(oc.depth_scale))
        filt = np.zeros_like(raw)
        rb.ref_bilateral(w, h, p(raw), p(filt))
        flat = np.zeros(sum(a * b for a, b in sizes), np.float32)
        cpu.ref_depth_pyramid(p(filt), w, h, 3, p(flat))
        lv, off = [], 0
        for a, b in sizes:
            lv.append(np.ascontiguousarray(flat[off:off + a * b]))
            off += a * b
        ok = 1
        if k > 0:
            ok, Tn = ref_track(rt, oc, lv, md, mv, mn, T, None)
            if ok:
                T = np.ascontiguousarray(Tn, np.float32)
        poses.append(T.copy())
        tracked.append(int(ok))
        if not ok:
            continue
        Ti = np.zeros(16, np.float32)
        m4.ref_inverse4(p(T), p(Ti))
        cam = np.zeros(3, np.float32)
        cu.ref_camera_center(p(T), p(cam))
        ri.ref_integrate_color(w, h, p(K0), p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(tsdf), p(wt),
                               p(col), p(raw), p(rgb), p(T), p(Ti), None)
        for l, (a, b) in enumerate(sizes):
            img = np.zeros(a * b, np.uint8)
            rr.ref_render_icp(w, h, p(K0), l, p(dims), p(org), p(cen), oc.voxel_size, oc.mu, oc.max_w, p(tsdf),
                              p(wt), p(T), p(Ti), p(cam), p(np.array([0, 0, -1], np.float32)), p(md[l]), p(mv[l]),
                              p(mn[l]), p(img))
    return np.stack(poses), np.array(tracked, np.int32), tsdf, wt, md, mv, mn


def refpin_pipeline():
    """four 120x90 frames through the reference's own stages (about a minute:
    the tracker's block trees run as cooperative threads)"""
    if O.load_ref_pin_gpu() is None or O.load_ref_pin_cpu() is None:
        raise SystemExit("the reference tree is not mounted; refpin_pipeline.npz cannot be regenerated")
    oc, dmm = pipeline_case()
    poses, tracked, tsdf, wt, md, mv, mn = ref_pipeline(oc, dmm)
    np.savez_compressed(os.path.join(OUT, "refpin_pipeline.npz"), depth_mm=dmm, poses=poses, tracked=tracked,
                        weight=wt, depth0=md[0], vertex0=mv[0], normal0=mn[0])


def refpin_gpu_config(c):
    """or_config of the refpin_gpu case: float TSDF storage (the reference's)"""
    oc = O.OrConfig()
    oc.width, oc.height = int(c["width"]), int(c["height"])
    oc.fx, oc.fy, oc.cx, oc.cy = float(c["fx"]), float(c["fy"]), float(c["cx"]), float(c["cy"])
    oc.levels = 3
    for k in range(3):
        oc.dim[k] = int(c["dim"])
        oc.origin[k] = float(c["origin"][k])
        oc.icp_iters[k] = (10, 5, 4)[k]
    oc.voxel_size, oc.mu, oc.max_w = float(c["voxel_size"]), float(c["mu"]), float(c["max_w"])
    oc.th_icp, oc.cos_normal, oc.tsdf_store, oc.reduce_mode, oc.depth_scale = 0.01, -3.0, 0, 1, 0.001
    return oc


if __name__ == "__main__":
    refpin()
    refpin_cuda()
    refpin_gpu()
    refpin_track()
    refpin_cpu()
    refpin_pipeline()
    seq_small()
    print("fixtures written to", OUT)

"""The oracle's primitives against the reference's own math.

STAC/Util/_yooji_math_inlines.h (pose algebra) builds on Linux from the
reference tree as it is; STAC/Util/_yooji_cuda_math.h (the per-pixel and
per-voxel helpers: 6x6 Cholesky, bilinear map lookups, camera and voxel
geometry) builds as host C++ with the stand-ins of oracle/ref_shim/ for the
CUDA qualifiers and InfiniTAM's vector types.  Their outputs on fixed inputs
are committed in tests/golden/refpin.npz and refpin_cuda.npz (written by
tests/golden/gen_golden.py), and where the tree is mounted the harnesses are
also rebuilt and compared live."""
import ctypes
import os

import numpy as np
import pytest

import oracle_py as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin.npz")


def test_se3_exp_matches_reference_bit_for_bit(built):
    g = np.load(GOLD)
    for xi, e in zip(g["xi"], g["exp"]):
        assert np.array_equal(O.se3_exp(xi).reshape(16), e)


def test_inverse4_matches_reference_bit_for_bit(built):
    g = np.load(GOLD)
    for m, inv in zip(g["mats"], g["inv"]):
        assert np.array_equal(O.pose_inverse(m).reshape(16), inv)


def test_fp64_exp_agrees_with_reference_to_float_precision(built):
    g = np.load(GOLD)
    for xi, e in zip(g["xi"], g["exp"]):
        d = O.se3_exp(xi.astype(np.float64), f64=True).reshape(16)
        assert np.max(np.abs(d - e.astype(np.float64))) < 2e-6


def test_live_reference_harness(built):
    ref = O.load_ref_pin()
    if ref is None:
        pytest.skip("reference tree not mounted on this host")
    rng = np.random.default_rng(5)
    for _ in range(200):
        xi = (rng.standard_normal(6) * 10.0 ** rng.uniform(-5, -0.5)).astype(np.float32)
        e = np.empty(16, np.float32)
        ref.ref_se3_exp(xi.ctypes.data_as(ctypes.c_void_p), e.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(O.se3_exp(xi).reshape(16), e)
        m = e.copy()
        m[3], m[7], m[11] = rng.uniform(-1, 1, 3).astype(np.float32)
        inv = np.empty(16, np.float32)
        ref.ref_inverse4(m.ctypes.data_as(ctypes.c_void_p), inv.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(O.pose_inverse(m).reshape(16), inv)


# ---- the reference's _yooji_cuda_math.h helpers -----------------------------
GOLD_CUDA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin_cuda.npz")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_cholesky_factor_and_solve_match_reference_bit_for_bit(built):
    """d_lld_LL_Decomposition / d_sls_Solve_Linear_System_using_LLD, including
    singular systems (a zero pivot fails the solve) and a negative pivot
    (the square root's NaN spreads through the factor)"""
    g = np.load(GOLD_CUDA)
    lib = O.load()
    assert (g["ok"] == 0).any() and (g["ok"] == 1).any()
    for A, rhs, L_ref, x_ref, ok in zip(g["A"], g["rhs"], g["L"], g["x"], g["ok"]):
        L = np.zeros(36, np.float32)
        lib.or_prim_cholesky6(_p(np.ascontiguousarray(A)), _p(L))
        assert np.array_equal(_bits(L), _bits(L_ref))
        x = np.zeros(6, np.float32)
        assert lib.or_prim_chol_solve6(_p(np.ascontiguousarray(L_ref)), _p(np.ascontiguousarray(rhs)), _p(x)) == ok
        if ok:
            assert np.array_equal(_bits(x), _bits(x_ref))


def test_bilinear_map_lookups_match_reference_bit_for_bit(built):
    """d_giv / d_gin: -100 sentinels reject, taps with zero weight are not
    read, the normal form is normalised"""
    g = np.load(GOLD_CUDA)
    lib = O.load()
    w, h, mp = int(g["w"]), int(g["h"]), np.ascontiguousarray(g["map"])
    for k, (norm, ref_out, ref_ok) in enumerate(((0, g["giv"], g["giv_ok"]), (1, g["gin"], g["gin_ok"]))):
        assert (ref_ok == 0).any() and (ref_ok == 1).any()
        for (xf, yf), r, ok in zip(g["xy"], ref_out, ref_ok):
            o = np.zeros(3, np.float32)
            assert lib.or_prim_bilinear3(float(xf), float(yf), w, h, _p(mp), norm, _p(o)) == ok
            if ok:
                assert np.array_equal(_bits(o), _bits(r)), (k, xf, yf)


def test_camera_and_voxel_geometry_match_reference_bit_for_bit(built):
    """d_p_Project, d_bp_Back_Project, d_t_Transform, d_r_Rotate,
    d_gcc_Get_Camera_Center, d_gpv / d_gpw"""
    g = np.load(GOLD_CUDA)
    lib = O.load()
    dim = np.ascontiguousarray(g["dim"])
    for i in range(len(g["K"])):
        K, p3, T = (np.ascontiguousarray(g[k][i]) for k in ("K", "p3", "T"))
        uv = np.zeros(2, np.float32)
        lib.or_prim_project(_p(p3), _p(K), _p(uv))
        assert np.array_equal(_bits(uv), _bits(g["proj"][i]))
        u, v, d = (float(t) for t in g["uvd"][i])
        b = np.zeros(3, np.float32)
        lib.or_prim_back_project(u, v, _p(K), d, _p(b))
        assert np.array_equal(_bits(b), _bits(g["bproj"][i]))
        for rot, key in ((0, "trans"), (1, "rot")):
            o = np.zeros(3, np.float32)
            lib.or_prim_transform(_p(p3), _p(T), rot, _p(o))
            assert np.array_equal(_bits(o), _bits(g[key][i]))
        c = np.zeros(3, np.float32)
        lib.or_camera_center(_p(T), _p(c))
        assert np.array_equal(_bits(c), _bits(g["cen"][i]))
        org, q, vox = (np.ascontiguousarray(g[k][i]) for k in ("org", "q", "vox"))
        o = np.zeros(3, np.float32)
        assert lib.or_prim_pos_in_voxel(_p(q), _p(org), _p(dim), float(g["inv"][i]), _p(o)) == g["gpv_ok"][i]
        assert np.array_equal(_bits(o), _bits(g["gpv"][i]))
        lib.or_prim_pos_in_world(_p(vox), _p(org), float(g["inv"][i]), _p(o))
        assert np.array_equal(_bits(o), _bits(g["gpw"][i]))


def test_live_reference_device_math(built):
    """where the reference tree is mounted: fresh random systems and lookups
    against the header compiled from it"""
    ref = O.load_ref_pin_cuda()
    if ref is None:
        pytest.skip("reference tree not mounted on this host")
    lib = O.load()
    rng = np.random.default_rng(7)
    for it in range(100):
        M = rng.standard_normal((6, 6)).astype(np.float32) * np.float32(10.0 ** rng.uniform(-3, 3))
        A = np.ascontiguousarray((M @ M.T).astype(np.float32).reshape(36))
        L1, L2 = np.zeros(36, np.float32), np.zeros(36, np.float32)
        ref.ref_lld6(_p(A), _p(L1))
        lib.or_prim_cholesky6(_p(A), _p(L2))
        assert np.array_equal(_bits(L1), _bits(L2))
        b = rng.standard_normal(6).astype(np.float32)
        x1, x2 = np.zeros(6, np.float32), np.zeros(6, np.float32)
        assert ref.ref_sls6(_p(L1), _p(b), _p(x1)) == lib.or_prim_chol_solve6(_p(L1), _p(b), _p(x2))
        assert np.array_equal(_bits(x1), _bits(x2))
    w, h = 17, 11
    for it in range(300):
        mp = rng.standard_normal((h, w, 3)).astype(np.float32)
        mp[rng.random((h, w)) < 0.1] = -100.0
        mp = np.ascontiguousarray(mp.reshape(-1))
        xf, yf = float(np.float32(rng.uniform(-0.5, w - 0.5))), float(np.float32(rng.uniform(-0.5, h - 0.5)))
        for norm, fn in ((0, ref.ref_giv), (1, ref.ref_gin)):
            o1, o2 = np.zeros(3, np.float32), np.zeros(3, np.float32)
            r1 = fn(xf, yf, w, h, _p(mp), _p(o1))
            assert r1 == lib.or_prim_bilinear3(xf, yf, w, h, _p(mp), norm, _p(o2))
            if r1:
                assert np.array_equal(_bits(o1), _bits(o2))


# ---- the reference's renderer and integrator, run as host code ----------------
GOLD_GPU = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin_gpu.npz")


def _gpu_case_config(g):
    sys_path_golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    import sys
    if sys_path_golden not in sys.path:
        sys.path.insert(0, sys_path_golden)
    import gen_golden
    return gen_golden.refpin_gpu_config(dict(width=int(g["cfg_w"]), height=int(g["cfg_h"]), fx=float(g["cfg_f"]),
                                             fy=float(g["cfg_f"]), cx=int(g["cfg_w"]) / 2.0, cy=int(g["cfg_h"]) / 2.0,
                                             dim=int(g["cfg_dim"]), origin=g["cfg_origin"],
                                             voxel_size=float(g["cfg_vox"]), mu=float(g["cfg_mu"]),
                                             max_w=float(g["cfg_maxw"])))


def test_integration_and_raycast_match_the_reference_kernels_bit_for_bit(built):
    """The oracle's TSDF / weight / colour update and its ray-cast maps equal
    those of the reference's own g_fvsc + g_ctvc and g_rmi kernels (their
    sources run as host code), frame by frame and level by level.  The
    colour image has no zero texel and the depth frame a zero border, so
    every colour sample interpolates (where one cannot, the reference blends
    an uninitialised value and the oracle keeps the colour)."""
    g = np.load(GOLD_GPU)
    oc = _gpu_case_config(g)
    vol = O.Volume(oc)
    for k in range(2):
        T = g["T"][k]
        vol.integrate_color(g["depth"][k], g["rgb"][k], T, O.pose_inverse(T))
        t, w = vol.get()
        assert np.array_equal(w, g["weight"][k].astype(np.uint16)), k
        assert np.array_equal(_bits(t), _bits(g["tsdf"][k])), k
        assert np.array_equal(vol.get_color().reshape(-1), g["colour"][k]), k
    T = g["T"][2]
    cam = O.camera_center(T)
    for l in range(3):
        d, v, n, img = vol.raycast(l, T, O.pose_inverse(T), cam, np.array([0, 0, -1], np.float32))
        assert (d > 0).sum() > 20
        assert np.array_equal(_bits(d.reshape(-1)), _bits(g["depth%d" % l])), l
        assert np.array_equal(_bits(v.reshape(-1)), _bits(g["vertex%d" % l])), l
        assert np.array_equal(_bits(n.reshape(-1)), _bits(g["normal%d" % l])), l
        assert np.array_equal(img.reshape(-1), g["img%d" % l]), l


def _check_variant(var, has_v, got, ref):
    """got: the oracle's (depth, vertex, normals, image, colour); ref: the
    reference's arrays.  Variant 0 (scene maps, nearest-voxel colour) keeps
    the reference's red plane out of it: there the reference writes green
    (z_yooji_cuda_tsdf_renderer.cu:185,1418), the oracle the true red"""
    d, v, n, img, rgb = got
    assert np.array_equal(_bits(d.reshape(-1)), _bits(ref["depth"])), var
    assert np.array_equal(_bits(n.reshape(-1)), _bits(ref["normal"])), var
    assert np.array_equal(img.reshape(-1), ref["img"]), var
    if has_v:
        assert np.array_equal(_bits(v.reshape(-1)), _bits(ref["vertex"])), var
    rgb, rref = rgb.reshape(3, -1), ref["rgb"].reshape(3, -1)
    if var == 0:
        assert np.array_equal(rref[0], rref[1])
        assert np.array_equal(rgb[1:], rref[1:])
        assert (rgb[0] != rgb[1]).sum() > 0
    else:
        assert np.array_equal(rgb, rref), var


def test_scene_renders_and_carving_match_the_reference_kernels_bit_for_bit(built):
    """the oracle's three other renders against the reference's
    rmis_Render_Maps_for_Scene (with and without a vertex map) and the
    vertex-less rmi_Render_Maps_for_ICP, and its carving against
    uvv_Update_Valid_Volume after a third integration"""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import gen_golden
    g = np.load(GOLD_GPU)
    oc = _gpu_case_config(g)
    vol = O.Volume(oc)
    for k in range(2):
        T = g["T"][k]
        vol.integrate_color(g["depth"][k], g["rgb"][k], T, O.pose_inverse(T))
    T = g["T"][2]
    Ti, cam = O.pose_inverse(T), O.camera_center(T)
    light = np.array([0, 0, -1], np.float32)
    for var, (mode, level, has_v) in gen_golden.RENDER_VARIANTS.items():
        got = vol.render_variant(mode, level, T, Ti, cam, light, vertex=has_v, color=True)
        assert (got[0] > 0).sum() > 100
        ref = {k: g["var%d_%s" % (var, k)] for k in ("depth", "normal", "img", "rgb") + (("vertex",) if has_v else ())}
        _check_variant(var, has_v, got, ref)
    vol.integrate_color(g["carve_depth"], g["carve_rgb"], T, Ti)
    assert vol.update_valid_volume(gen_golden.carve_mask(int(g["cfg_dim"]))) > 20
    t, w = vol.get()
    assert np.array_equal(w, g["carve_weight"].astype(np.uint16))
    assert np.array_equal(_bits(t), _bits(g["carve_tsdf"]))
    assert np.array_equal(vol.get_color().reshape(-1), g["carve_colour"])


def test_live_reference_kernels(built):
    """where the reference tree is mounted: a 160x120 sequence into a 96^3 cube,
    the oracle against the reference's renderer and integrator run live"""
    libs = O.load_ref_pin_gpu()
    if libs is None:
        pytest.skip("reference tree not mounted on this host")
    rr, ri, rt, rb = libs
    import vs_scanner as V

    w, h, dim = 160, 120, 96
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=4, seed=5, dropout_iid=0.01)
    depth_mm, rgb, gt, centre = V.synth_generate_rgb(sc)
    origin, vox = V.cube_around(centre, 0.75, dim)
    oc = _gpu_case_config(dict(cfg_w=w, cfg_h=h, cfg_f=f, cfg_dim=dim, cfg_origin=np.array(origin, np.float32),
                               cfg_vox=vox, cfg_mu=0.03, cfg_maxw=100.0))
    geo = np.zeros(5, np.float32)
    O.load().or_config_geometry(ctypes.byref(oc), _p(geo))
    K0 = np.array([oc.fx, oc.fy, oc.cx, oc.cy], np.float32)
    dims, org, cen = np.array([dim] * 3, np.int32), np.array(list(oc.origin), np.float32), np.ascontiguousarray(geo[:3])
    n = dim ** 3
    t_ref, w_ref, c_ref = np.ones(n, np.float32), np.zeros(n, np.uint8), np.zeros(3 * n, np.uint8)
    vol = O.Volume(oc)
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import gen_golden
    mask = gen_golden.carve_mask(dim)
    for k in range(3):
        raw = np.ascontiguousarray(O.depth_to_m(depth_mm[k]), np.float32)
        raw[0, :] = raw[-1, :] = raw[:, 0] = raw[:, -1] = 0.0
        img = np.ascontiguousarray(np.maximum(rgb[k], 1), np.uint8)
        T = np.ascontiguousarray(gt[k], np.float32)
        Ti = np.ascontiguousarray(O.pose_inverse(T))
        vol.integrate_color(raw, img, T, Ti)
        if k == 2:
            assert vol.update_valid_volume(mask) > 100
        ri.ref_integrate_color(w, h, _p(K0), _p(dims), _p(org), _p(cen), oc.voxel_size, oc.mu, oc.max_w, _p(t_ref),
                               _p(w_ref), _p(c_ref), _p(raw), _p(img), _p(T), _p(Ti), _p(mask) if k == 2 else None)
        t, wt = vol.get()
        assert np.array_equal(wt, w_ref.astype(np.uint16)) and np.array_equal(_bits(t), _bits(t_ref)), k
        assert np.array_equal(vol.get_color().reshape(-1), c_ref), k
    T = np.ascontiguousarray(gt[3], np.float32)
    Ti = np.ascontiguousarray(O.pose_inverse(T))
    cam = np.ascontiguousarray(O.camera_center(T), np.float32)
    light = np.array([0, 0, -1], np.float32)
    t, wt = vol.get()
    for l in range(3):
        lw, lh = w >> l, h >> l
        d, v, nn, im = (np.zeros(lw * lh, np.float32), np.zeros(3 * lw * lh, np.float32),
                        np.zeros(3 * lw * lh, np.float32), np.zeros(lw * lh, np.uint8))
        rr.ref_render_icp(w, h, _p(K0), l, _p(dims), _p(org), _p(cen), oc.voxel_size, oc.mu, oc.max_w,
                          _p(np.ascontiguousarray(t)), _p(wt.astype(np.uint8)), _p(T), _p(Ti), _p(cam), _p(light),
                          _p(d), _p(v), _p(nn), _p(im))
        od, ov, on, oi = vol.raycast(l, T, Ti, cam, light)
        assert (d > 0).sum() > 300 >> (2 * l)
        for a, b in ((od, d), (ov, v), (on, nn)):
            assert np.array_equal(_bits(a.reshape(-1)), _bits(b)), l
        assert np.array_equal(oi.reshape(-1), im), l
        if l == 0:
            for var, (mode, vlev, has_v) in gen_golden.RENDER_VARIANTS.items():
                vw, vh = w >> vlev, h >> vlev
                ref = {"depth": np.zeros(vw * vh, np.float32), "vertex": np.zeros(3 * vw * vh, np.float32),
                       "normal": np.zeros(3 * vw * vh, np.float32), "img": np.zeros(vw * vh, np.uint8),
                       "rgb": np.zeros(3 * vw * vh, np.uint8)}
                rr.ref_render_variant(var, w, h, _p(K0), vlev, _p(dims), _p(org), _p(cen), oc.voxel_size, oc.mu,
                                      oc.max_w, _p(np.ascontiguousarray(t)), _p(wt.astype(np.uint8)), _p(c_ref), _p(T),
                                      _p(Ti), _p(cam), _p(light), *(_p(ref[k]) for k in ("depth", "vertex", "normal",
                                                                                          "img", "rgb")))
                got = vol.render_variant(mode, vlev, T, Ti, cam, light, vertex=has_v, color=True)
                assert (got[0] > 0).sum() > 300 >> (2 * vlev)
                _check_variant(var, has_v, got, ref)
            # the per-pixel ICP term of the next frame against these maps
            icp = _icp_case(np.ascontiguousarray(O.depth_to_m(depth_mm[3]), np.float32))
            ATA, ATb, ok = np.zeros((w * h, 36), np.float32), np.zeros((w * h, 6), np.float32), np.zeros(w * h, np.uint8)
            rt.ref_icp_terms(w, h, _p(K0), _p(icp["depth"]), _p(d), _p(v), _p(nn), _p(icp["T21"]), 0.01, _p(ATA),
                             _p(ATb), _p(ok))
            assert ok.sum() > 200
            _check_icp_terms(w, h, K0, icp["depth"], v, nn, icp["T21"], ATA, ATb, ok)


def _icp_case(depth):
    import sys
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    if d not in sys.path:
        sys.path.insert(0, d)
    import gen_golden
    return gen_golden.icp_case(depth)


def _check_icp_terms(w, h, K, depth, vtx, nrm, T21, ATA, ATb, ok):
    """the oracle's per-pixel A, b give the reference's ATA = A A^T and
    ATb = A b (each product rounded once, in float32) and the same pixels"""
    lib = O.load()
    A, b = np.zeros(6, np.float32), np.zeros(1, np.float32)
    args = [_p(np.ascontiguousarray(a, np.float32)) for a in (K, depth, vtx, nrm, T21)]
    for y in range(h):
        for x in range(w):
            i = y * w + x
            r = lib.or_prim_icp_term(x, y, w, h, *args[:4], args[4], 0.01, _p(A), _p(b))
            assert r == ok[i], (x, y)
            if r:
                assert np.array_equal(_bits(np.outer(A, A).astype(np.float32).reshape(-1)), _bits(ATA[i])), (x, y)
                assert np.array_equal(_bits((A * b[0]).astype(np.float32)), _bits(ATb[i])), (x, y)


def test_icp_terms_match_the_reference_kernel_bit_for_bit(built):
    """the per-pixel term of the reference's d_cssfp (z_yooji_cuda_pose_tracker.cu:279-395)
    against level-1 model maps the reference rendered"""
    g = np.load(GOLD_GPU)
    w, h = int(g["cfg_w"]) >> 1, int(g["cfg_h"]) >> 1
    assert g["icp_ok"].sum() > 20
    _check_icp_terms(w, h, g["icp_K"], g["icp_depth"], g["vertex1"], g["normal1"], g["icp_T21"], g["icp_ATA"],
                     g["icp_ATb"], g["icp_ok"])


def test_bilateral_matches_the_reference_kernel_bit_for_bit(built):
    """the oracle's bilateral filter against the reference's d_bilateral_filter
    (z_yooji_cuda_img_proc.cu:103-141, run as host code with the documented
    texture-fetch rules for its linear-filtered texture) on a frame with
    single zero texels, 2x2 holes, zero lines and a depth step"""
    g = np.load(GOLD_GPU)
    w, h = int(g["cfg_w"]), int(g["cfg_h"])
    x = np.ascontiguousarray(g["bil_in"], np.float32)
    out = np.zeros_like(x)
    O.load().or_bilateral(_p(x), w, h, _p(out))
    assert (g["bil_out"] == 0).sum() > 100 and (g["bil_out"] > 0).sum() > 2000
    assert np.array_equal(_bits(out), _bits(g["bil_out"]))


def test_live_reference_bilateral(built):
    """where the reference tree is mounted: ragged and VGA frames"""
    libs = O.load_ref_pin_gpu()
    if libs is None:
        pytest.skip("reference tree not mounted on this host")
    rb = libs[3]
    import vs_scanner as V

    for (w, h, seed) in ((97, 75, 3), (170, 130, 4), (640, 480, 5)):
        f = 285.0 * w / 320.0
        sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=1, seed=seed, dropout_iid=0.02)
        d = V.synth_generate(sc)[0]
        x = _bilateral_input(O.depth_to_m(d[0]))
        a, b = np.zeros_like(x), np.zeros_like(x)
        rb.ref_bilateral(w, h, _p(x), _p(a))
        O.load().or_bilateral(_p(x), w, h, _p(b))
        assert np.array_equal(_bits(a), _bits(b)), (w, h)


def _bilateral_input(depth):
    import sys
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    if d not in sys.path:
        sys.path.insert(0, d)
    import gen_golden
    return gen_golden.bilateral_input(depth)


# ---- the reference's whole tracker (tp_Track_Pose) ----------------------------
GOLD_TRACK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin_track.npz")


def _gen_golden():
    import sys
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    if d not in sys.path:
        sys.path.insert(0, d)
    import gen_golden
    return gen_golden


def test_tracking_matches_the_reference_tracker_bit_for_bit(built):
    """the oracle's ICP in the reference's reduction mode (16x16 block trees of
    all 36 + 6 sums, block partials summed serially in float) against the
    reference's tp_Track_Pose (z_yooji_cuda_pose_tracker.cu:790-1042, with
    g_glsbw :548-697 run as cooperative block threads): the tracked pose over
    the three levels, and over level 0 from an identity initial increment"""
    g = np.load(GOLD_TRACK)
    oc, dmm, gt, ind, md, mv, mn = _gen_golden().track_case(int(g["w"]), int(g["h"]))
    assert np.array_equal(dmm, g["depth_mm"]) and np.array_equal(gt, g["gt"])
    for init, ok_key, T_key in ((None, "ok_levels", "T_levels"), (np.eye(4, dtype=np.float32), "ok_init", "T_init")):
        ok, T, info = O.track(oc, ind, mv, mn, gt[1], init_T12=init)
        assert ok and bool(g[ok_key])
        assert np.array_equal(_bits(T), _bits(g[T_key])), T_key
    # a converging case: closer to the true pose of frame 2 than the start
    import helpers
    assert helpers.camera_centre_err(g["T_levels"], gt[2]) < 0.5 * helpers.camera_centre_err(gt[1], gt[2])


def test_live_reference_tracker(built):
    """where the reference tree is mounted: 80x60 from an identity increment
    (level 0, ten iterations) and over the three levels, where the 20x15 level
    gives too few correspondences and both fail"""
    libs = O.load_ref_pin_gpu()
    if libs is None:
        pytest.skip("reference tree not mounted on this host")
    G = _gen_golden()
    oc, dmm, gt, ind, md, mv, mn = G.track_case(80, 60, dim=64)
    for init in (np.eye(4, dtype=np.float32), None):
        rok, rT = G.ref_track(libs[2], oc, ind, md, mv, mn, gt[1], init)
        ok, T, info = O.track(oc, ind, mv, mn, gt[1], init_T12=init)
        assert bool(rok) == ok
        if ok:
            assert np.array_equal(_bits(T), _bits(rT))
        else:
            assert np.array_equal(rT, gt[1])  # the reference leaves the pose


# ---- the reference's CPU image processor (pyramid, point / normal maps) ------
GOLD_CPU = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin_cpu.npz")


def _check_cpu_maps(depth0, K0, ref_levels, ref_K, ref_vtx, ref_nrm):
    """the oracle's pyramid (sdg5 + ddh), level intrinsics (dih) and point /
    normal maps (cpm + enm, with the in-place rejection) against the
    reference's"""
    lib = O.load()
    Kl = np.zeros(12, np.float32)
    lib.or_level_intrinsics(_p(np.ascontiguousarray(K0, np.float32)), 3, _p(Kl))
    assert np.array_equal(_bits(Kl), _bits(ref_K.reshape(-1)))
    lv = [np.ascontiguousarray(depth0, np.float32)]
    for l in range(1, 3):
        lv.append(np.ascontiguousarray(O.pyramid_down(lv[-1]), np.float32))
        assert np.array_equal(_bits(lv[l]), _bits(ref_levels[l])), l
    for l in range(3):
        v, n = O.point_normal_map(lv[l], Kl[4 * l:4 * l + 4].copy())
        assert np.array_equal(_bits(v), _bits(ref_vtx[l])), l
        assert np.array_equal(_bits(n), _bits(ref_nrm[l])), l
    # the rejection recurrence is exercised: more invalid points than holes
    assert (ref_vtx[0][..., 0] == -100).sum() > (lv[0] <= 0).sum()
    assert (ref_nrm[0][..., 0] != -100).sum() > 300


def test_pyramid_and_input_maps_match_the_reference_bit_for_bit(built):
    """the reference's cpdd_Construct_Pyramids_Down_Depth, cpm_Compute_Point_Map,
    enm_Estimate_Normal_Map and dih_Downsample_Intrinsics_Half
    (z_yooji_image_processor.cpp:119-227,368-407,567-612,857-937), taken
    unchanged from the reference tree over stand-ins for the KAISION types"""
    g = np.load(GOLD_CPU)
    _check_cpu_maps(g["depth0"], g["K0"], [g["pyr%d" % l] for l in range(3)], g["K"],
                    [g["vertex%d" % l] for l in range(3)], [g["normal%d" % l] for l in range(3)])


def test_registration_matches_the_reference_bit_for_bit(built):
    """the oracle's depth -> colour warp against the reference's
    z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates (z_yooji_object_scanner.cpp:2429-2476)
    with convert_pixel_coord (z_yooji_matrix_rgbd.cpp:101-118)"""
    g = np.load(GOLD_CPU)
    h, w = g["depth0"].shape
    out = O.warp_depth(g["depth0"], g["K0"], g["warp_T"], g["warp_Kr"], w, h)
    assert (g["warp"] > 0).mean() > 0.5
    assert np.array_equal(_bits(out), _bits(g["warp"]))


def test_live_reference_pyramid_and_input_maps(built):
    """where the reference tree is mounted: ragged, QVGA and VGA frames"""
    lib = O.load_ref_pin_cpu()
    if lib is None:
        pytest.skip("reference tree not mounted on this host")
    G = _gen_golden()
    for (w, h, seed) in ((97, 75, 3), (320, 240, 4), (640, 480, 5)):
        x, K0 = G.cpu_case(w, h, seed)
        _check_cpu_maps(x, K0, *G.ref_cpu_maps(lib, x, K0))
        # registration into a colour camera of the same size and of twice the size
        T, Kr = G.warp_rig(w, h)
        for (wr, hr, K) in ((w, h, Kr), (2 * w, 2 * h, Kr * np.float32(2))):
            ref = np.zeros((hr, wr), np.float32)
            lib.ref_warp_depth(_p(x), w, h, _p(K0), _p(T), _p(np.ascontiguousarray(K)), wr, hr, _p(ref))
            assert (ref > 0).sum() > 0.2 * w * h
            assert np.array_equal(_bits(O.warp_depth(x, K0, T, K, wr, hr)), _bits(ref)), (w, h, wr)


# ---- the whole per-frame path, chained from the reference's own stages -------
GOLD_PIPE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin_pipeline.npz")


def _check_pipeline(oc, dmm, poses, tracked, weight, depth0, vertex0, normal0):
    s = O.Session(oc)
    for k in range(dmm.shape[0]):
        assert s.frame(dmm[k]) == bool(tracked[k]), k
        assert np.array_equal(_bits(s.pose()), _bits(poses[k])), k
    _, w = s.volume().get()
    assert np.array_equal(w, weight.astype(np.uint16))
    m = s.maps(0)
    assert (depth0 > 0).sum() > 1000
    assert np.array_equal(_bits(m["model_depth"]), _bits(depth0.reshape(m["model_depth"].shape)))
    assert np.array_equal(_bits(m["model_vertex"]), _bits(vertex0.reshape(m["model_vertex"].shape)))
    assert np.array_equal(_bits(m["model_normal"]), _bits(normal0.reshape(m["model_normal"].shape)))


def test_whole_frame_loop_matches_the_reference_stages_bit_for_bit(built):
    """four frames through the oracle's session (its own stage order) against
    the same frames through the reference's own bilateral filter, pyramid,
    tracker, integrator and renderer chained in the reference scanner's order:
    every pose, the tracked flags, the final weights and the final level-0
    model maps are identical"""
    g = np.load(GOLD_PIPE)
    oc, dmm = _gen_golden().pipeline_case()
    assert np.array_equal(dmm, g["depth_mm"])
    assert g["tracked"].all()
    _check_pipeline(oc, dmm, g["poses"], g["tracked"], g["weight"], g["depth0"], g["vertex0"], g["normal0"])


def test_live_whole_frame_loop(built):
    """where the reference tree is mounted: three 80x60 frames into a 64^3
    cube, a case whose rays sample within one voxel of the cube's low faces
    (where ITMMath's toInt decides the trilinear taps)"""
    if O.load_ref_pin_gpu() is None or O.load_ref_pin_cpu() is None:
        pytest.skip("reference tree not mounted on this host")
    G = _gen_golden()
    oc, dmm = G.pipeline_case(w=80, h=60, dim=64, frames=3, seed=8)
    poses, tracked, tsdf, wt, md, mv, mn = G.ref_pipeline(oc, dmm)
    _check_pipeline(oc, dmm, poses, tracked, wt, md[0], mv[0], mn[0])

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

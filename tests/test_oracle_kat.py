"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden files for this path, so the oracle is
pinned by closed-form cases built from the reference's own formulas, and by
the reference's host math compiled from source (test_refpin.py)."""
import numpy as np
import pytest

import oracle_py as O


def test_bilateral_constant_field_unchanged(built):
    d = np.full((24, 32), 1.2345, np.float32)
    out = O.bilateral(d)
    assert np.max(np.abs(out - d)) <= 2e-7


def test_bilateral_single_zero_texel_is_averaged_not_a_hole(built):
    # taps are means of 2x2 texels, so one zero texel pulls its neighbours
    # toward 0 but never makes a tap <= 0 (z_yooji_cuda_img_proc.cu:119-128)
    d = np.full((20, 20), 1.0, np.float32)
    d[10, 10] = 0.0
    out = O.bilateral(d)
    assert np.all(out > 0)
    assert out[10, 10] < 1.0


def test_bilateral_2x2_zero_block_makes_5x5_hole(built):
    d = np.full((24, 24), 1.0, np.float32)
    d[10:12, 10:12] = 0.0  # the tap at (11, 11) reads four zero texels
    out = O.bilateral(d)
    hole = out == 0.0
    ys, xs = np.nonzero(hole)
    assert hole.sum() == 25
    assert (ys.min(), ys.max(), xs.min(), xs.max()) == (9, 13, 9, 13)


def test_bilateral_border_taps_clamp(built):
    # a zero column at x = 0: the tap at X = 0 reads texels {clamp(-1), 0} = {0, 0}
    d = np.full((16, 16), 1.0, np.float32)
    d[:, 0] = 0.0
    out = O.bilateral(d)
    assert np.all(out[:, :3] == 0.0)  # taps X in [x-2, x+2] reach X = 0 for x <= 2
    assert np.all(out[:, 3:] > 0.0)


def test_gaussian_table_matches_reference_formula(built):
    g = np.zeros(5, np.float32)
    O.load().or_gaussian_table(4.0, 2, g.ctypes.data_as(O.ctypes.c_void_p))
    x = np.arange(-2, 3, dtype=np.float32)
    assert np.allclose(g, np.exp(-(x * x) / np.float32(32.0)), rtol=0, atol=1e-7)


def test_pyramid_constant_field(built):
    d = np.ones((32, 40), np.float32)
    l1 = O.pyramid_down(d)
    assert l1.shape == (16, 20)
    # kept pixel (2i+1, 2j+1) is smoothed when 2 <= 2i+1 < W-2, else 0
    assert np.all(l1[1:-1, 1:-1] == 1.0)
    assert np.all(l1[0, :] == 0) and np.all(l1[-1, :] == 0)
    assert np.all(l1[:, 0] == 0) and np.all(l1[:, -1] == 0)


def test_pyramid_mixes_zero_depth(built):
    # no validity mask (z_yooji_image_processor.cpp:904-928): zeros are averaged in
    d = np.ones((32, 32), np.float32)
    d[15, 15] = 0.0
    l1 = O.pyramid_down(d)
    assert l1[7, 7] == pytest.approx(1.0 - 36.0 / 256.0)


def test_level_intrinsics_halving(built):
    cfg = O.make_config(640, 480, 525.0, 525.0, 319.5, 239.5, 64, (0, 0, 0), 0.01, 0.02)
    K = O.level_K(cfg)
    f32 = np.float32
    assert K[1, 0] == f32(262.5) and K[2, 0] == f32(131.25)
    assert K[1, 2] == f32(0.5) * (f32(319.5) - f32(0.5))
    assert K[2, 3] == f32(0.5) * (K[1, 3] - f32(0.5))


def test_point_normal_map_plane_facing_camera(built):
    K = np.array([100.0, 100.0, 16.0, 12.0], np.float32)
    d = np.full((24, 32), 0.8, np.float32)
    v, n = O.point_normal_map(d, K)
    assert np.allclose(v[5, 7], [0.8 * (7 - 16) / 100, 0.8 * (5 - 12) / 100, 0.8], atol=1e-7)
    inner = n[1:-1, 1:-1].reshape(-1, 3)
    assert np.allclose(inner, [0, 0, -1], atol=1e-6)
    assert np.all(n[0] == -100) and np.all(n[:, 0] == -100)


def test_point_normal_map_steep_plane_rejection_alternates(built):
    # a plane tilted ~70 deg: every interior normal fails -n_z >= cos 60.  The
    # reference rewrites the point map in place on rejection
    # (z_yooji_image_processor.cpp:216-219), so along a row rejected and
    # skipped pixels alternate: only every other pixel is rejected.
    K = np.array([100.0, 100.0, 16.0, 12.0], np.float32)
    ys, xs = np.mgrid[0:24, 0:32].astype(np.float32)
    x = (xs - 16) / 100
    d = (1.0 / (1.0 - 2.5 * x)).astype(np.float32)  # plane z = 1 + 2.5 X
    v, n = O.point_normal_map(d, K)
    assert np.all(n[1:-1, 1:-1] == -100)  # no normal survives
    row = v[1, 1:-1, 0] == -100  # vertices invalidated only where rejected
    assert row[0] and not row[1] and row[2] and not row[3]
    # the row below: a pixel under a rejected one is blocked (not rejected)
    row2 = v[2, 1:-1, 0] == -100
    assert not row2[0] and row2[1] and not row2[2]


def test_se3_exp_zero_and_inverse(built):
    assert np.array_equal(O.se3_exp(np.zeros(6)), np.eye(4, dtype=np.float32))
    xi = np.array([0.01, -0.02, 0.015, 0.05, -0.01, 0.02])
    T = O.se3_exp(xi, f64=True)
    assert np.allclose(T[:3, :3] @ T[:3, :3].T, np.eye(3), atol=1e-14)
    Ti = O.pose_inverse(T.astype(np.float32))
    assert np.allclose(Ti @ T.astype(np.float32), np.eye(4), atol=1e-6)


def _plane_case(dim=64, d=0.6, mu=0.03):
    # camera at the origin looking down +z, plane z = d; voxel centres on the
    # optical axis project exactly onto the principal point (cx, cy integral)
    vox = np.float32(1.0 / 64)
    k = dim // 2
    origin = (-(k + 0.5) * float(vox), -(k + 0.5) * float(vox), 0.3)
    cfg = O.make_config(64, 48, 60.0, 60.0, 32.0, 24.0, dim, origin, float(vox), mu, levels=1,
                        icp_iters=(1, 0, 0), tsdf_store=0, reduce_mode=3)
    return cfg, np.full((48, 64), d, np.float32), k


def test_integrate_plane_closed_form(built):
    cfg, depth, k = _plane_case()
    vol = O.Volume(cfg)
    I = np.eye(4, dtype=np.float32)
    vol.integrate(depth, I, I)
    t, w = vol.get()
    t = t.reshape(64, 64, 64)
    w = w.reshape(64, 64, 64)
    vox = np.float32(cfg.voxel_size)
    for z in range(64):
        zc = (np.float32(z) + np.float32(0.5)) / (np.float32(1) / vox) + np.float32(0.3)
        sdf = np.float32(0.6) - zc
        active = abs(zc - 0.6) <= 5 * 0.03  # sub-cube activation band (-4 mu .. +1 mu, 8-voxel bricks)
        if sdf < -np.float32(0.03):
            assert w[z, k, k] == 0
        elif active and w[z, k, k]:
            assert t[z, k, k] == pytest.approx(min(1.0, float(sdf) / 0.03), abs=2e-6)
    # voxels right at the surface are always updated
    zs = int(round((0.6 - 0.3) / float(vox) - 0.5))
    assert w[zs, k, k] == 1


def test_raycast_plane(built):
    cfg, depth, k = _plane_case()
    vol = O.Volume(cfg)
    I = np.eye(4, dtype=np.float32)
    for _ in range(3):
        vol.integrate(depth, I, I)
    dep, v, n, img = vol.raycast(0, I, I, np.zeros(3, np.float32))
    c = dep[20:28, 28:36]
    assert np.all(np.abs(c - 0.6) < 1e-3)
    # the ray-distance SDF of off-axis voxels bends the field slightly
    assert np.allclose(n[20:28, 28:36].reshape(-1, 3), [0, 0, -1], atol=1e-2)


def test_icp_same_frame_converges_at_first_iteration(built):
    # model maps equal to the back-projected input: b = 0, so x = 0 and every
    # level stops after one iteration
    rng = np.random.default_rng(0)
    h, w = 48, 64
    K = np.array([60.0, 60.0, 32.0, 24.0], np.float32)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float32)
    depth = (1.0 + 0.2 * np.sin(xs / 7.0) * np.cos(ys / 5.0)).astype(np.float32)
    cfg = O.make_config(w, h, 60.0, 60.0, 32.0, 24.0, 64, (0, 0, 0), 0.01, 0.03, levels=1,
                        icp_iters=(10, 0, 0), reduce_mode=3, th_icp=0.01)
    v, _ = O.point_normal_map(depth, K)
    # analytic-ish normals: finite differences of the vertex map, all valid
    dx = np.gradient(v, axis=1)
    dy = np.gradient(v, axis=0)
    nrm = np.cross(dx, dy)
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    vv = v.copy()
    ok, T, info = O.track(cfg, [depth], [vv], [nrm.astype(np.float32)], np.eye(4), f64=True)
    assert ok
    assert info[0] == 1
    assert np.allclose(T, np.eye(4), atol=1e-6)
    del rng


def _corner_depth(T_gc, K, w, h):
    """depth of three orthogonal planes x = -0.4, y = 0.3, z = 1.2 (global frame)
    seen from pose T_gc; returns depth and the per-pixel plane normal (camera frame)"""
    T = np.asarray(T_gc, np.float64)
    Tcg = np.linalg.inv(T)
    C = Tcg[:3, 3]
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    dc = np.stack([(xs - K[2]) / K[0], (ys - K[3]) / K[1], np.ones_like(xs)], -1)
    dg = dc @ Tcg[:3, :3].T
    planes = [(np.array([1.0, 0, 0]), -0.4), (np.array([0, 1.0, 0]), 0.3), (np.array([0, 0, 1.0]), 1.2)]
    best = np.full((h, w), np.inf)
    nb = np.zeros((h, w, 3))
    for nrm, off in planes:
        den = dg @ nrm
        t = (off - C @ nrm) / np.where(np.abs(den) < 1e-12, np.nan, den)
        t = np.where(t > 0, t, np.inf)
        sel = t < best
        best = np.where(sel, t, best)
        nc = T[:3, :3] @ nrm
        if nc @ (T[:3, :3] @ (np.array([0, 0, 0]) - C)) < 0:
            pass
        nb[sel] = nc
    # orient normals towards the camera (negative z in the camera frame)
    flip = nb[..., 2] > 0
    nb[flip] *= -1
    return best.astype(np.float32), nb.astype(np.float32)


def test_icp_recovers_known_twist(built):
    w, h = 80, 60
    K = np.array([70.0, 70.0, 40.0, 30.0], np.float32)
    xi = np.array([0.004, -0.006, 0.003, 0.006, -0.004, 0.008])
    T1 = O.se3_exp(xi, f64=True)  # T_gc of frame 1 (frame 0 at identity)
    d0, n0 = _corner_depth(np.eye(4), K, w, h)
    d1, _ = _corner_depth(T1, K, w, h)
    v0, _ = O.point_normal_map(d0, K)
    valid = np.isfinite(d0)
    v0[~valid] = -100
    n0[~valid] = -100
    d1 = np.where(np.isfinite(d1), d1, 0).astype(np.float32)
    cfg = O.make_config(w, h, 70.0, 70.0, 40.0, 30.0, 64, (0, 0, 0), 0.01, 0.03, levels=1,
                        icp_iters=(20, 0, 0), reduce_mode=3, th_icp=0.05 ** 2)
    ok, T, info = O.track(cfg, [d1], [v0], [n0], np.eye(4), f64=True)
    assert ok
    assert np.degrees(np.arccos(np.clip((np.trace(T[:3, :3].T @ T1[:3, :3]) - 1) / 2, -1, 1))) < np.degrees(1e-4)
    assert np.linalg.norm(T[:3, 3] - T1[:3, 3]) < 1e-4

"""Scene-mode ray-casts and the object-mode render without a vertex map
(rmis_Render_Maps_for_Scene, rmi_Render_Maps_for_ICP's second form), and
valid-volume carving (uvv_Update_Valid_Volume), against the CPU oracle.

The render variants use the tolerance of the ICP ray-cast parity test
(vertices within 1 mm on 99.9 % of the pixels both hit, hit masks agreeing on
99.9 %); colour and shaded images are equal wherever both agree.  Carving is
integer work on identical volumes: the sub-cubes reset, the weights and the
colours are bit-identical, the TSDF within the integration test's bound."""
import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V

LIGHT = np.array([0, 0, -1], np.float32)


def _plane_volume(ocfg, plane=40.3):
    """every voxel weight 1, TSDF of a plane z = plane (voxels), positive in
    front (smaller z), one TSDF unit per mu as integration makes it"""
    X, Y, Z = ocfg.dim[0], ocfg.dim[1], ocfg.dim[2]
    z = np.arange(Z, dtype=np.float32)
    band = ocfg.mu / ocfg.voxel_size
    q = np.rint(np.clip((plane - z) / band, -1, 1) * 32767.0) / 32767.0
    t = np.broadcast_to(q[:, None, None], (Z, Y, X)).astype(np.float32).ravel()
    return t, np.ones(X * Y * Z, np.uint16)


# ---- oracle known answers (CPU) -------------------------------------------
def test_oracle_scene_raycast_from_inside_the_volume():
    """a camera inside the cube looking along +z at a plane: the scene ray-cast
    (from the camera centre, no cone) hits it at the plane's depth, with the
    global normal (0, 0, -1) and full shading; the object ray-cast (a segment
    through the bounding sphere centred on the camera's far side) is not the
    one the reference uses there"""
    c = helpers.make_case(width=80, height=60, dim=64, size=1.0, frames=1, seed=2)
    ocfg = c["ocfg"]
    vol = O.Volume(ocfg)
    plane = 40.3
    vol.set(*_plane_volume(ocfg, plane))
    org = np.array(ocfg.origin[:3], np.float64)
    vs = float(ocfg.voxel_size)
    cam = org + vs * (np.array([31.5, 31.5, 10.5]) + 0.5)  # voxel (31.5, 31.5, 10.5) (centres at i + 0.5)
    Tgc = np.eye(4, dtype=np.float32)
    Tgc[:3, 3] = -cam.astype(np.float32)
    Tcg = O.pose_inverse(Tgc)
    mode = O.RAY_SCENE | O.RAY_GLOBAL_NORMALS | O.RAY_NEAREST_COLOR
    dep, v, n, img, _ = vol.render_variant(mode, 0, Tgc, Tcg, cam.astype(np.float32), LIGHT)
    hit = dep > 0
    assert hit.mean() > 0.95
    want = (plane + 0.5 - (10.5 + 0.5)) * vs  # surface at voxel z plane + 0.5 (world = (i + 0.5) vs + origin)
    # the last step overshoots by < 1 voxel; each of the two corrections of
    # 0.9 mu TSDF along a ray at angle a to the normal leaves (1 - 0.9 cos a)
    # of it: < 0.07 voxel at this image's corners
    assert np.allclose(dep[hit], want, atol=0.1 * vs), (dep[hit].min(), dep[hit].max(), want)
    assert np.allclose(n[hit], [0, 0, -1], atol=1e-4)
    assert (img[hit] == 255).all()
    assert np.allclose(v[hit][:, 2], dep[hit])
    # no hit: depth 0, vertex / normal -100, image 0
    assert (n[~hit] == -100).all() and (img[~hit] == 0).all()


def test_oracle_render_view_white_background_and_global_normals():
    c = helpers.make_case(width=80, height=60, dim=64, size=1.0, frames=2, seed=2)
    vol = O.Volume(c["ocfg"])
    T = np.eye(4, dtype=np.float32)
    raw = O.depth_to_m(c["depth"][0])
    vol.integrate_color(raw, np.full((3, 60, 80), 77, np.uint8), T, T)
    Tgc = c["gt"][1].astype(np.float32)
    Tcg = O.pose_inverse(Tgc)
    cam = O.camera_center(Tgc)
    od, ov, on, oi, orgb = vol.raycast_color(0, Tgc, Tcg, cam, LIGHT)
    mode = O.RAY_GLOBAL_NORMALS | O.RAY_WHITE_BACKGROUND
    dep, v, n, img, rgb = vol.render_variant(mode, 0, Tgc, Tcg, cam, LIGHT, vertex=False, color=True)
    assert v is None
    assert np.array_equal(dep, od)
    hit = dep > 0
    assert hit.sum() > 300 and (~hit).sum() > 300
    # camera-frame normals of the ICP maps are the global ones rotated
    R = Tgc[:3, :3]
    assert np.allclose(on[hit], n[hit] @ R.T, atol=1e-5)
    assert (rgb[:, ~hit] == 255).all()
    assert np.array_equal(rgb[:, hit], orgb[:, hit])


def test_oracle_carving_resets_flagged_empty_subcubes_only():
    c = helpers.make_case(width=80, height=60, dim=64, size=1.0, frames=2, seed=2)
    ocfg = c["ocfg"]
    X, Y, Z = ocfg.dim[0], ocfg.dim[1], ocfg.dim[2]
    vol = O.Volume(ocfg)
    T = np.eye(4, dtype=np.float32)
    vol.integrate(O.depth_to_m(c["depth"][0]), T, T)
    t0, w0 = vol.get()
    flags = vol.flags().astype(bool)
    nsx, nsy, nsz = X // 8, Y // 8, Z // 8
    # valid: the half-space x < X/2, plus one voxel in an otherwise invalid sub-cube
    valid = np.zeros((Z, Y, X), np.uint8)
    valid[:, :, : X // 2] = 1
    fl = flags.reshape(nsz, nsy, nsx)
    keep = np.argwhere(fl[:, :, nsx // 2 + 1:])[0]
    kz, ky, kx = keep[0], keep[1], keep[2] + nsx // 2 + 1
    valid[kz * 8 + 3, ky * 8 + 4, kx * 8 + 5] = 1
    sc_valid = valid.reshape(nsz, 8, nsy, 8, nsx, 8).any(axis=(1, 3, 5))
    expect = fl & ~sc_valid
    assert expect.sum() > 5 and (fl & sc_valid).sum() > 5
    n = vol.update_valid_volume(valid)
    assert n == expect.sum()
    t1, w1 = vol.get()
    vox_sc = np.zeros((Z, Y, X), bool)
    vox_sc[:] = np.repeat(np.repeat(np.repeat(expect, 8, 0), 8, 1), 8, 2)
    reset = vox_sc.ravel()
    assert (w1[reset] == 0).all() and (t1[reset] == 1.0).all()
    assert np.array_equal(w1[~reset], w0[~reset]) and np.array_equal(t1[~reset], t0[~reset])
    assert (w0[reset] > 0).any()
    # the sub-cube with one valid voxel is kept whole
    assert fl[kz, ky, kx] and not expect[kz, ky, kx]
    # unflagged: a second carving finds nothing
    assert np.array_equal(vol.flags().astype(bool).reshape(nsz, nsy, nsx), fl & sc_valid)
    assert vol.update_valid_volume(valid) == 0


# ---- GPU parity ------------------------------------------------------------
def _dev(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _zeros(n, dtype):
    torch = pytest.importorskip("torch")
    return torch.zeros(n, dtype=dtype, device="cuda")


@pytest.fixture(scope="module")
def ccase(gpu):
    import test_color

    return test_color.color_case(frames=4)


def _coloured_volume(cc, frames=3):
    vol = O.Volume(cc["ocfg"])
    for k in range(frames):
        raw = O.depth_to_m(cc["depth"][k])
        Tgc = cc["gt"][k].astype(np.float32)
        vol.integrate_color(raw, cc["rgb"][k], Tgc, O.pose_inverse(Tgc))
    return vol


def _compare(od, ov, on, oi, orgb, gd, gv, gn, gi, grgb):
    valid_o, valid_g = od > 0, gd > 0
    same = valid_o == valid_g
    assert same.mean() >= 0.999, same.mean()
    both = valid_o & valid_g
    assert both.sum() > 1000
    if ov is not None:
        err = np.linalg.norm(gv[both] - ov[both], axis=1)
        assert (err <= 1e-3).mean() >= 0.999, np.percentile(err, 99.9)
        assert (gv[~valid_g] == -100).all()
    assert np.percentile(np.abs(gn[both] - on[both]).max(1), 99.9) < 1e-3
    assert (np.abs(gi[same].astype(int) - oi[same].astype(int)) <= 1).mean() >= 0.999
    if orgb is not None:
        # colour of a surface point within the ray-cast tolerance: within one
        # level on 99.9 % of the pixels
        dc = np.abs(grgb.astype(np.int32) - orgb.astype(np.int32))[:, same]
        assert (dc.max(axis=0) <= 1).mean() >= 0.999


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["scene_maps", "scene_view", "view"])
def test_render_variants_identical_volume(gpu, ccase, variant):
    torch = pytest.importorskip("torch")
    vol = _coloured_volume(ccase)
    t, w = vol.get()
    ocol = vol.get_color()
    Tgc = ccase["gt"][3].astype(np.float32)
    Tcg = O.pose_inverse(Tgc)
    cam = O.camera_center(Tgc)
    mode, level, has_v = {
        "scene_maps": (O.RAY_SCENE | O.RAY_GLOBAL_NORMALS | O.RAY_NEAREST_COLOR, 0, True),
        "scene_view": (O.RAY_SCENE | O.RAY_GLOBAL_NORMALS, 0, False),
        "view": (O.RAY_GLOBAL_NORMALS | O.RAY_WHITE_BACKGROUND, 1, False),
    }[variant]
    od, ov, on, oi, orgb = vol.render_variant(mode, level, Tgc, Tcg, cam, LIGHT, vertex=has_v, color=True)
    with V.Session(ccase["cfg"]) as s:
        s.set_volume(t, w)
        s.set_color_volume(ocol)
        lw, lh = s.levels[level][0], s.levels[level][1]
        d_gc, d_cg = _dev(Tgc), _dev(Tcg)
        gd, gn = _zeros(lw * lh, torch.float32), _zeros(3 * lw * lh, torch.float32)
        gv = _zeros(3 * lw * lh, torch.float32) if has_v else None
        gi, grgb = _zeros(lw * lh, torch.uint8), _zeros(3 * lw * lh, torch.uint8)
        m0 = s.maps(0)["model_depth"].copy()
        if variant == "view":
            s.rmi_render_view(level, d_gc.data_ptr(), d_cg.data_ptr(), cam, LIGHT, gd.data_ptr(), gn.data_ptr(),
                              gi.data_ptr(), grgb.data_ptr())
        else:
            s.rmis_render_maps_for_scene(d_gc.data_ptr(), d_cg.data_ptr(), cam, LIGHT, gd.data_ptr(),
                                         gv.data_ptr() if has_v else None, gn.data_ptr(), gi.data_ptr(),
                                         grgb.data_ptr())
        # the session's own model maps are untouched
        assert np.array_equal(s.maps(0)["model_depth"], m0)
    gd = gd.cpu().numpy().reshape(lh, lw)
    gn = gn.cpu().numpy().reshape(lh, lw, 3)
    gv = gv.cpu().numpy().reshape(lh, lw, 3) if has_v else None
    gi = gi.cpu().numpy().reshape(lh, lw)
    grgb = grgb.cpu().numpy().reshape(3, lh, lw)
    _compare(od, ov, on, oi, orgb, gd, gv, gn, gi, grgb)
    hit = gd > 0
    if variant == "view":
        assert (grgb[:, ~hit] == 255).all()
    else:
        assert (grgb[:, ~hit] == 0).all()
        assert (grgb[0][hit] > 0).mean() > 0.9


@pytest.mark.gpu
def test_scene_render_without_colour_volume_rejects_colour_output(gpu):
    torch = pytest.importorskip("torch")
    c = helpers.make_case(width=160, height=120, dim=64, size=1.0, frames=1, seed=2)
    T = np.eye(4, dtype=np.float32)
    with V.Session(c["cfg"]) as s:
        d_t = _dev(T)
        n = 160 * 120
        gd, gn, gi = _zeros(n, torch.float32), _zeros(3 * n, torch.float32), _zeros(n, torch.uint8)
        grgb = _zeros(3 * n, torch.uint8)
        with pytest.raises(V.VsError) as e:
            s.rmis_render_maps_for_scene(d_t.data_ptr(), d_t.data_ptr(), np.zeros(3, np.float32), LIGHT,
                                         gd.data_ptr(), None, gn.data_ptr(), gi.data_ptr(), grgb.data_ptr())
        assert e.value.code == V.VS_ERR_STATE
        # without colour it runs
        s.rmis_render_maps_for_scene(d_t.data_ptr(), d_t.data_ptr(), np.zeros(3, np.float32), LIGHT,
                                     gd.data_ptr(), None, gn.data_ptr(), gi.data_ptr(), None)


def _half_mask(cfg, axis=2, frac=0.55):
    X, Y, Z = cfg.dim[0], cfg.dim[1], cfg.dim[2]
    m = np.zeros((Z, Y, X), np.uint8)
    cut = int(frac * (Z, Y, X)[axis])
    sl = [slice(None)] * 3
    sl[axis] = slice(0, cut)
    m[tuple(sl)] = 1
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("device_mask", [False, True])
def test_carving_matches_oracle(gpu, ccase, device_mask):
    cfg = ccase["cfg"]
    vol = O.Volume(ccase["ocfg"])
    valid = _half_mask(cfg)
    with V.Session(cfg) as s:
        for k in range(3):
            raw = O.depth_to_m(ccase["depth"][k])
            Tgc = ccase["gt"][k].astype(np.float32)
            Tcg = O.pose_inverse(Tgc)
            vol.integrate_color(raw, ccase["rgb"][k], Tgc, Tcg)
            d = [_dev(a) for a in (raw, ccase["rgb"][k], Tgc, Tcg)]
            s.cdtocc_convert_depth_to_tsdf_color(*(x.data_ptr() for x in d))
            if k == 1:
                # carve between integrations: the next frame re-activates and refills
                dm = _dev(valid) if device_mask else None
                ng = s.uvv_update_valid_volume(dm.data_ptr() if device_mask else valid)
                no = vol.update_valid_volume(valid)
                assert ng == no and no > 0
                assert s.uvv_update_valid_volume(valid) == 0 == vol.update_valid_volume(valid)
        ng = s.uvv_update_valid_volume(valid)
        no = vol.update_valid_volume(valid)
        assert ng == no and no > 0
        t, w = s.volume()
        col = s.color_volume()
        act = np.sort(s.active_bricks())
    ot, ow = vol.get()
    assert np.array_equal(w, ow)
    assert np.array_equal(col, vol.get_color())
    m = ow > 0
    assert np.max(np.abs(helpers.q16(t[m]) - helpers.q16(ot[m]))) <= 1
    assert (t[~m] == 1.0).all()
    # the carved side is empty where the last frame's sub-cubes were reset
    assert act.size > 0


@pytest.mark.gpu
def test_carving_after_scan_frames_resets_last_frame_subcubes(gpu, ccase):
    """per-frame path: the flagged set is the last frame's active sub-cubes;
    the carving resets exactly those of them without a valid voxel, and the
    ray-cast and integration of later frames see the carved volume"""
    cfg = ccase["cfg"]
    X, Y, Z = cfg.dim[0], cfg.dim[1], cfg.dim[2]
    valid = _half_mask(cfg, axis=0, frac=0.5)
    nsx, nsy, nsz = X // 8, Y // 8, Z // 8
    sc_valid = valid.reshape(nsz, 8, nsy, 8, nsx, 8).any(axis=(1, 3, 5)).ravel()
    with V.Session(cfg) as s:
        for k in range(3):
            s.set_color_frame(ccase["rgb"][k])
            s.scan_frame_host(ccase["depth"][k])
        t0, w0 = s.volume()
        act = s.active_bricks().astype(np.int64)
        expect = act[~sc_valid[act]]
        assert expect.size > 0 and expect.size < act.size
        assert s.uvv_update_valid_volume(valid) == expect.size
        t1, w1 = s.volume()
        b = np.zeros(nsx * nsy * nsz, bool)
        b[expect] = True
        reset = np.repeat(np.repeat(np.repeat(b.reshape(nsz, nsy, nsx), 8, 0), 8, 1), 8, 2).ravel()
        assert (w1[reset] == 0).all() and (t1[reset] == 1.0).all()
        assert np.array_equal(w1[~reset], w0[~reset]) and np.array_equal(t1[~reset], t0[~reset])
        col = s.color_volume()
        assert (col[:, reset] == 0).all()
        # a later frame tracks and integrates on the carved volume
        s.set_color_frame(ccase["rgb"][3])
        _, tracked = s.scan_frame_host(ccase["depth"][3])
        assert tracked


@pytest.mark.gpu
def test_snapshot_keeps_the_flagged_set(gpu, ccase, tmp_path):
    """a session saved after its frames and loaded again carves the same
    sub-cubes as the session that kept running"""
    cfg = ccase["cfg"]
    valid = _half_mask(cfg, axis=1, frac=0.5)
    path = str(tmp_path / "c.vssnap")
    with V.Session(cfg) as a:
        for k in range(3):
            a.set_color_frame(ccase["rgb"][k])
            a.scan_frame_host(ccase["depth"][k])
        a.save(path)
        na = a.uvv_update_valid_volume(valid)
        ta, wa = a.volume()
        ca = a.color_volume()
    b = V.Session.load(path)
    try:
        assert b.uvv_update_valid_volume(valid) == na > 0
        tb, wb = b.volume()
        assert np.array_equal(wa, wb) and np.array_equal(ta, tb)
        assert np.array_equal(ca, b.color_volume())
    finally:
        b.close()

"""Colour integration and colour ray-cast (the reference's g_ctvc colour branch
and d_grvi), against the CPU oracle.

On identical inputs the colour volume after integration and the colour image
of the ray-cast are bit-identical (8-bit values from the same float
operations); colour never changes tracking, and a colour session gives the
same colour alone and in a batch."""
import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V


def color_case(width=160, height=120, dim=96, size=0.75, frames=4, seed=5):
    f = 285.0 * width / 320.0
    sc = V.synth_config(width, height, fx=f, fy=f, cx=width / 2.0, cy=height / 2.0, n_frames=frames, seed=seed,
                        dropout_iid=0.01)
    depth, rgb, gt, centre = V.synth_generate_rgb(sc)
    origin, vox = V.cube_around(centre, size, dim)
    cfg = V.default_config(width, height, fx=f, fy=f, cx=width / 2.0, cy=height / 2.0, dim=(dim,) * 3,
                           origin=origin, voxel_size=vox, mu=0.03, color=1)
    return dict(depth=depth, rgb=rgb, gt=gt, cfg=cfg, ocfg=O.config_from_vs(cfg))


# ---- oracle known answers (CPU) -------------------------------------------
def test_oracle_color_of_a_uniform_volume_is_that_colour():
    """a volume whose every voxel has weight 1 and one colour ray-casts to that
    colour wherever the ray hits (toUChar rounding of an exact interpolation)"""
    c = helpers.make_case(width=80, height=60, dim=64, size=1.0, frames=1, seed=2)
    ocfg = c["ocfg"]
    vol = O.Volume(ocfg)
    raw = O.depth_to_m(c["depth"][0])
    T = np.eye(4, dtype=np.float32)
    vol.integrate(raw, T, T)
    t, w = vol.get()
    w[:] = 1
    vol.set(t, w)
    n = ocfg.dim[0] * ocfg.dim[1] * ocfg.dim[2]
    vol.set_color(np.stack([np.full(n, 17), np.full(n, 128), np.full(n, 250)]).astype(np.uint8))
    dep, _, _, _, rgb = vol.raycast_color(0, T, T, O.camera_center(T))
    hit = dep > 0
    assert hit.sum() > 500
    assert (rgb[0][hit] == 17).all() and (rgb[1][hit] == 128).all() and (rgb[2][hit] == 250).all()
    assert (rgb[:, ~hit] == 0).all()


def test_oracle_first_blend_takes_the_sample():
    """weight 0 -> the first update stores the sample, truncated to 8 bits;
    a constant image gives that constant or one below (the interpolation of a
    constant can round just under it).  Voxels projecting within half a pixel
    of the right or bottom border update depth (nearest pixel) but cannot be
    interpolated, so their colour stays 0."""
    c = helpers.make_case(width=80, height=60, dim=64, size=1.0, frames=1, seed=2)
    vol = O.Volume(c["ocfg"])
    raw = O.depth_to_m(c["depth"][0])
    T = np.eye(4, dtype=np.float32)
    rgb = np.stack([np.full((60, 80), 90), np.full((60, 80), 91), np.full((60, 80), 200)]).astype(np.uint8)
    vol.integrate_color(raw, rgb, T, T)
    _, w = vol.get()
    col = vol.get_color()
    upd = w > 0
    assert upd.sum() > 1000
    for k, v in enumerate((90, 91, 200)):
        assert set(np.unique(col[k][upd])) <= {0, v - 1, v}
        assert (col[k][upd] > 0).mean() > 0.95
    assert (col[:, ~upd] == 0).all()


# ---- GPU parity ------------------------------------------------------------
@pytest.fixture(scope="module")
def ccase(gpu):
    return color_case()


def _dev(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_color_integrate_identical_inputs(gpu, ccase):
    cfg = ccase["cfg"]
    vol = O.Volume(ccase["ocfg"])
    with V.Session(cfg) as s:
        for k in range(4):
            raw = O.depth_to_m(ccase["depth"][k])
            Tgc = ccase["gt"][k].astype(np.float32)
            Tcg = O.pose_inverse(Tgc)
            vol.integrate_color(raw, ccase["rgb"][k], Tgc, Tcg)
            d_raw, d_rgb, d_gc, d_cg = _dev(raw), _dev(ccase["rgb"][k]), _dev(Tgc), _dev(Tcg)
            s.cdtocc_convert_depth_to_tsdf_color(d_raw.data_ptr(), d_rgb.data_ptr(), d_gc.data_ptr(),
                                                 d_cg.data_ptr())
        t, w = s.volume()
        col = s.color_volume()
    ot, ow = vol.get()
    ocol = vol.get_color()
    assert np.array_equal(w, ow)
    assert np.array_equal(col, ocol)
    assert (col[:, w > 0] > 0).mean() > 0.9


@pytest.mark.gpu
def test_color_raycast_identical_volume(gpu, ccase):
    torch = pytest.importorskip("torch")
    vol = O.Volume(ccase["ocfg"])
    for k in range(3):
        raw = O.depth_to_m(ccase["depth"][k])
        Tgc = ccase["gt"][k].astype(np.float32)
        vol.integrate_color(raw, ccase["rgb"][k], Tgc, O.pose_inverse(Tgc))
    t, w = vol.get()
    ocol = vol.get_color()
    Tgc = ccase["gt"][3].astype(np.float32)
    Tcg = O.pose_inverse(Tgc)
    cam = O.camera_center(Tgc)
    light = np.array([0, 0, -1], np.float32)
    with V.Session(ccase["cfg"]) as s:
        s.set_volume(t, w)
        s.set_color_volume(ocol)
        assert np.array_equal(s.color_volume(), ocol)
        d_gc, d_cg = _dev(Tgc), _dev(Tcg)
        for l, (lw, lh, *_k) in enumerate(s.levels):
            od, _, _, _, orgb = vol.raycast_color(l, Tgc, Tcg, cam, light)
            gd = torch.zeros(lw * lh, dtype=torch.float32, device="cuda")
            gv = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gn = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gi = torch.zeros(lw * lh, dtype=torch.uint8, device="cuda")
            grgb = torch.zeros(3 * lw * lh, dtype=torch.uint8, device="cuda")
            s.rmi_render_maps_color(l, d_gc.data_ptr(), d_cg.data_ptr(), cam, light, gd.data_ptr(), gv.data_ptr(),
                                    gn.data_ptr(), gi.data_ptr(), grgb.data_ptr())
            grgb = grgb.cpu().numpy().reshape(3, lh, lw)
            gd = gd.cpu().numpy().reshape(lh, lw)
            same = (gd > 0) == (od > 0)
            assert same.mean() >= 0.999
            # the trilinear colour at a surface point within the ray-cast
            # tolerance of the oracle's: within one level on 99.9 % of pixels
            dc = np.abs(grgb.astype(np.int32) - orgb.astype(np.int32))[:, same]
            assert (dc.max(axis=0) <= 1).mean() >= 0.999, l
            assert (grgb[0][gd > 0] > 0).mean() > 0.9


@pytest.mark.gpu
def test_color_frames_leave_tracking_unchanged_and_batch_equals_alone(gpu, ccase):
    cfg = ccase["cfg"]
    plain = V.default_config(cfg.width, cfg.height)
    for f, _ in V.VsConfig._fields_:
        setattr(plain, f, getattr(cfg, f))
    plain.color = 0
    with V.Session(cfg) as a, V.Session(plain) as p:
        for k in range(4):
            a.set_color_frame(ccase["rgb"][k])
            a.scan_frame_host(ccase["depth"][k])
            p.scan_frame_host(ccase["depth"][k])
        assert np.array_equal(a.pose()[1], p.pose()[1])
        assert np.array_equal(a.volume()[1], p.volume()[1])
        col_alone = a.color_volume()
        map_alone = a.color_map(0)
        assert (map_alone[0][a.maps(0)["model_depth"] > 0] > 0).mean() > 0.9
        plain_pose, plain_maps = p.pose()[1], [p.maps(l)["model_vertex"] for l in range(plain.levels)]
    # a batch holding colour sessions and a session without colour: the colour
    # ray-cast's two launches serve all three, each as alone
    other = color_case(width=320, height=240, dim=64, size=1.0, frames=4, seed=6)
    with V.Session(cfg) as a, V.Session(other["cfg"]) as b, V.Session(plain) as q, V.Batch() as batch:
        for k in range(4):
            a.set_color_frame(ccase["rgb"][k])
            b.set_color_frame(other["rgb"][k])
            batch.step_host([a, b, q], [ccase["depth"][k], other["depth"][k], ccase["depth"][k]])
        assert np.array_equal(a.color_volume(), col_alone)
        assert np.array_equal(a.color_map(0), map_alone)
        assert np.array_equal(q.pose()[1], plain_pose)
        for l in range(plain.levels):
            assert np.array_equal(q.maps(l)["model_vertex"], plain_maps[l]), l

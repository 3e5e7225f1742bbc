"""Edge cases of the per-frame path: empty frames, ragged image sizes, a
session losing tracking inside a batch, and the largest volume and image the
library accepts.

An empty frame (no valid depth) gives the ICP nothing to sum: the reference's
Cholesky then fails on a zero pivot, the frame counts as lost, and nothing is
integrated.  Image sizes that are not multiples of the kernels' tiles must
give the oracle's results as any other size does."""
import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _same_pose(T, oT):
    return helpers.rot_err(T, oT) < 1e-4 and helpers.trans_err(T, oT) < 1e-4


def test_empty_frame_is_lost_like_the_oracle(gpu):
    c = helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=4, seed=21)
    frames = [c["depth"][0], c["depth"][1], np.zeros_like(c["depth"][2]), c["depth"][3]]
    osess = O.Session(c["ocfg"])
    with V.Session(c["cfg"]) as s:
        for k, f in enumerate(frames):
            w_before = s.volume()[1].copy()
            T, tracked = s.scan_frame_host(f)
            otracked = osess.frame(f)
            assert tracked == otracked, k
            assert _same_pose(T, osess.pose()), k
            if k == 2:
                assert not tracked
                # nothing integrated on a lost frame
                assert np.array_equal(s.volume()[1], w_before)
        assert tracked  # the next frame tracks again from the last good pose


@pytest.mark.parametrize("size", [(170, 130), (97, 75)])
def test_ragged_image_sizes_match_the_oracle(gpu, size):
    """every frame's tracking against the oracle's tracker on the session's
    own inputs, then the ray-cast of the session's volume at its pose against
    the oracle's ray-cast of the same volume, at every level"""
    w, h = size
    c = helpers.make_case(width=w, height=h, dim=96, size=0.75, frames=3, seed=22)
    # ingest, filter and pyramid at the ragged size
    with V.Session(c["cfg"]) as s:
        d = torch.from_numpy(np.ascontiguousarray(c["depth"][1]).view(np.int16)).cuda()
        s.stage_filter(d.data_ptr())
        ref = [O.bilateral(O.depth_to_m(c["depth"][1]))]
        for l in range(1, 3):
            ref.append(O.pyramid_down(ref[-1]))
        for l in range(3):
            got = s.maps(l)["input_depth"]
            assert got.shape == ref[l].shape and np.max(np.abs(got - ref[l])) <= 1e-5, l
    _, lost, final = helpers.reanchored_track_check(c["depth"], c["cfg"], 3)
    assert not lost
    vol = O.Volume(c["ocfg"])
    vol.set(*final["volume"])
    T = np.ascontiguousarray(final["pose"], np.float32)
    light = np.array([0, 0, -1], np.float32)
    for l, m in enumerate(final["maps"]):
        od, ov, on, oi = vol.raycast(l, T, O.pose_inverse(T), O.camera_center(T), light)
        assert m["model_depth"].shape == od.shape
        helpers.assert_maps_match(m["model_depth"], m["model_vertex"], m["model_normal"], m["model_img"], od, ov, on,
                                  oi, "level %d" % l)


def test_lost_session_in_a_batch_leaves_the_others_alone(gpu):
    a_case = helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=3, seed=23)
    b_case = helpers.make_case(width=320, height=240, dim=64, size=1.0, frames=3, seed=24)
    with V.Session(a_case["cfg"]) as a:
        for k in range(3):
            a.scan_frame_host(a_case["depth"][k])
        alone = a.pose()[1]
        alone_w = a.volume()[1]
    with V.Session(a_case["cfg"]) as a, V.Session(b_case["cfg"]) as b, V.Batch() as batch:
        for k in range(3):
            fb = b_case["depth"][k] if k != 1 else np.zeros_like(b_case["depth"][k])
            T, tracked = batch.step_host([a, b], [a_case["depth"][k], fb])
            if k == 1:
                assert list(tracked) == [True, False]
        assert np.array_equal(a.pose()[1], alone)
        assert np.array_equal(a.volume()[1], alone_w)


def test_largest_volume_and_image(gpu):
    """1024^3 voxels (4 GiB of int16+uint16) and a 2048-pixel-wide image run;
    one step more on either axis is refused"""
    w, h = 2048, 1536
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=2, seed=25)
    depth, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, 1.5, 1024)
    cfg = V.default_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=(1024, 1024, 1024), origin=origin,
                           voxel_size=vox, mu=0.02)
    with V.Session(cfg) as s:
        for k in range(2):
            T, tracked = s.scan_frame_host(depth[k])
            assert tracked
        assert helpers.camera_centre_err(T, gt[1]) < 5e-3
        md = s.maps(0)["model_depth"]
        assert (md > 0).mean() > 0.3
    for bad in ((1032, 1024, 1024), (1024, 1024, 1032)):
        cfg.dim[0], cfg.dim[1], cfg.dim[2] = bad
        with pytest.raises(V.VsError) as e:
            V.Session(cfg)
        assert e.value.code == V.VS_ERR_ARG
    wide = V.default_config(w + 8, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=(64, 64, 64), origin=origin,
                            voxel_size=vox * 16, mu=0.02)
    with pytest.raises(V.VsError) as e:
        V.Session(wide)
    assert e.value.code == V.VS_ERR_ARG


def test_full_size_vga_512_integration_and_raycast(gpu):
    """the plain VGA configuration at full size (640x480 frames, 512^3 int16
    volume over 1.5 m, mu 2 cm): two integrations at the true poses give the
    oracle's weights bit for bit and its TSDF within one int16 step, and the
    ray-cast of that volume gives the oracle's maps (99.9 % of the hit pixels
    agree, vertices within 1 mm) at every level"""
    torch = pytest.importorskip("torch")
    c = helpers.make_case(width=640, height=480, dim=512, size=1.5, frames=3, seed=26, mu=0.02)
    cfg, ocfg = c["cfg"], c["ocfg"]
    vol = O.Volume(ocfg)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    with V.Session(cfg) as s:
        for k in range(2):
            raw = O.depth_to_m(c["depth"][k])
            T = c["gt"][k].astype(np.float32)
            Ti = O.pose_inverse(T)
            vol.integrate(raw, T, Ti)
            d_raw, d_gc, d_cg = dev(raw), dev(T), dev(Ti)
            s.cdtoc_convert_depth_to_tsdf(d_raw.data_ptr(), d_gc.data_ptr(), d_cg.data_ptr())
        t, w = s.volume()
        ot, ow = vol.get()
        assert np.array_equal(w, ow)
        m = ow > 0
        assert m.sum() > 1_000_000
        assert np.max(np.abs(helpers.q16(t[m]) - helpers.q16(ot[m]))) <= 1
        T = c["gt"][2].astype(np.float32)
        Ti = O.pose_inverse(T)
        cam = O.camera_center(T)
        light = np.array([0, 0, -1], np.float32)
        d_gc, d_cg = dev(T), dev(Ti)
        for l, (lw, lh, *_k) in enumerate(s.levels):
            od, ov, on, oi = vol.raycast(l, T, Ti, cam, light)
            gd = torch.zeros(lw * lh, dtype=torch.float32, device="cuda")
            gv = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gn = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gi = torch.zeros(lw * lh, dtype=torch.uint8, device="cuda")
            s.rmi_render_maps_for_icp(l, d_gc.data_ptr(), d_cg.data_ptr(), cam, light, gd.data_ptr(), gv.data_ptr(),
                                      gn.data_ptr(), gi.data_ptr())
            gd = gd.cpu().numpy().reshape(lh, lw)
            gv = gv.cpu().numpy().reshape(lh, lw, 3)
            valid_o, valid_g = od > 0, gd > 0
            assert valid_o.sum() > 0.2 * lw * lh, l
            assert (valid_o == valid_g).mean() >= 0.999, l
            both = valid_o & valid_g
            err = np.linalg.norm(gv[both] - ov[both], axis=1)
            assert (err <= 1e-3).mean() >= 0.999, l


@pytest.mark.parametrize("case_seed", range(6))
def test_random_shapes_match_the_oracle(gpu, case_seed):
    """seeded random image sizes (odd widths and heights included), non-cubic
    volumes and every TSDF storage: two integrations at the true poses give the
    oracle's weights bit for bit and its TSDF (within one int16 step), and the
    ray-cast of that volume its model maps at every level.  (Tracking is left
    out: on some of these scenes a few hundred correspondences make the 6x6
    system so ill-conditioned that the float and FP64 oracles disagree too.)"""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1000 + case_seed)
    w, h = int(rng.integers(48, 400)), int(rng.integers(64, 300))
    dims = tuple(int(8 * rng.integers(6, 21)) for _ in range(3))
    store = [V.VS_TSDF_INT16, V.VS_TSDF_FP16, V.VS_TSDF_FP32][case_seed % 3]
    f = 285.0 * w / 320.0
    sc = V.synth_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, n_frames=2, seed=40 + case_seed)
    depth, gt, centre = V.synth_generate(sc)
    vox = 1.2 / min(dims)
    origin = [float(centre[k]) - 0.5 * dims[k] * vox for k in range(3)]
    cfg = V.default_config(w, h, fx=f, fy=f, cx=w / 2.0, cy=h / 2.0, dim=dims, origin=origin, voxel_size=vox,
                           mu=max(0.03, 3 * vox), tsdf_type=store)
    vol = O.Volume(O.config_from_vs(cfg))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    with V.Session(cfg) as s:
        for k in range(2):
            raw = O.depth_to_m(depth[k])
            T = gt[k].astype(np.float32)
            Ti = O.pose_inverse(T)
            vol.integrate(raw, T, Ti)
            d_raw, d_gc, d_cg = dev(raw), dev(T), dev(Ti)
            s.cdtoc_convert_depth_to_tsdf(d_raw.data_ptr(), d_gc.data_ptr(), d_cg.data_ptr())
        t, wt = s.volume()
        ot, ow = vol.get()
        assert np.array_equal(wt, ow), (w, h, dims)
        m = ow > 0
        assert m.sum() > 1000
        if store == V.VS_TSDF_INT16:
            assert np.max(np.abs(helpers.q16(t[m]) - helpers.q16(ot[m]))) <= 1
        else:
            helpers.assert_tsdf_within_one_step(t[m], ot[m])
        cam = O.camera_center(T)
        light = np.array([0, 0, -1], np.float32)
        for l, (lw, lh, *_k) in enumerate(s.levels):
            od, ov, on, oi = vol.raycast(l, T, Ti, cam, light)
            gd = torch.zeros(lw * lh, dtype=torch.float32, device="cuda")
            gv = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gn = torch.zeros(3 * lw * lh, dtype=torch.float32, device="cuda")
            gi = torch.zeros(lw * lh, dtype=torch.uint8, device="cuda")
            s.rmi_render_maps_for_icp(l, d_gc.data_ptr(), d_cg.data_ptr(), cam, light, gd.data_ptr(), gv.data_ptr(),
                                      gn.data_ptr(), gi.data_ptr())
            gd = gd.cpu().numpy().reshape(lh, lw)
            gv = gv.cpu().numpy().reshape(lh, lw, 3)
            assert ((od > 0) == (gd > 0)).mean() >= 0.999, (l, w, h, dims)
            both = (od > 0) & (gd > 0)
            if l == 0:
                assert both.sum() > 100, (w, h, dims)
            if both.any():
                assert (np.linalg.norm(gv[both] - ov[both], axis=1) <= 1e-3).mean() >= 0.999, (l, w, h, dims)

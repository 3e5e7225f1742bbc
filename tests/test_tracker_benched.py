"""The tracker exactly as the serving-mix benchmark runs it, against the oracle.

Configuration of every benchmark session: 20 degree input/model normal
rejection (the build's extension of d_cssfp, applied on both sides), 10 cm
distance threshold (th_icp = 0.01 m^2), ICP 10/5/4 iterations, compensated
(two-sum) FP32 reduction, int16 TSDF over a 1.5 m cube with truncation
mu = max(2 cm, 5 voxels) (the reference's own rule is 5 voxels,
VCL_Volume_Scanner_View.cpp:423), with the
three camera models of the mix (320x240 f = 285, 512x424 f = 365, 640x480
f = 525), Kinect-style noise, 1.5 % dropout in 8x8 blobs and depth cut at
2.5 m.  Reference tracker: tp_Track_Pose and d_cssfp
(STAC/Engine/GPU/z_yooji_cuda_pose_tracker.cu:279-395, 790-1042).

Two forms:

* re-anchored, per frame: at every frame of a sequence the GPU session's own
  state (model maps of the previous ray-cast, filtered input pyramid, input
  normals, previous pose) is handed to the oracle's tracker, and the GPU's
  tracked pose must be within 1e-4 rad and 0.1 mm of the oracle's, FP32
  (the reduction mode of the run) and FP64 alike.  The identical inputs keep
  earlier frames' differences out of the comparison.
* free-running: the 640x480 / 512^3 session for 30 frames against the FP64
  oracle pipeline run on the same frames; every frame tracked on both sides
  and the camera trajectories within 1 mm (RMS and per frame).
"""
import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

COS20 = float(np.cos(np.radians(20.0)))
CAMERAS = {"320x240": (320, 240, 285.0, 160.0, 120.0), "512x424": (512, 424, 365.0, 255.5, 211.5),
           "640x480": (640, 480, 525.0, 319.5, 239.5)}


def bench_case(size, dim, frames, seed, mu=None):
    """A benchmark session's frames and configuration; mu None: the
    benchmark's rule max(2 cm, 5 voxels)"""
    w, h, f, cx, cy = CAMERAS[size]
    sc = V.synth_config(w, h, fx=f, fy=f, cx=cx, cy=cy, n_frames=frames, seed=seed, dropout_blob=0.015,
                        max_depth=2.5)
    depth, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, 1.5, dim)
    cfg = V.default_config(w, h, fx=f, fy=f, cx=cx, cy=cy, dim=(dim,) * 3, origin=origin, voxel_size=vox,
                           mu=max(0.02, 5.0 * vox) if mu is None else mu, th_icp=0.01, cos_normal=COS20,
                           icp_iters=(10, 5, 4), tsdf_type=V.VS_TSDF_INT16, reduce_mode=V.VS_REDUCE_KAHAN)
    return depth, gt, cfg


@pytest.mark.parametrize("size,dim,frames,seed", [("320x240", 128, 12, 1500), ("512x424", 256, 12, 1501),
                                                  ("640x480", 384, 12, 1502), ("640x480", 512, 30, 2)])
def test_tracker_reanchored_per_frame(gpu, size, dim, frames, seed):
    depth, _, cfg = bench_case(size, dim, frames, seed)
    worst, _, final = helpers.reanchored_track_check(depth, cfg, frames)
    print("%s %d^3: worst per-frame difference %.2e rad, %.2e m" % (size, dim, worst[0], worst[1]))
    # every frame of the benchmark's configuration is well-conditioned here
    assert not final["ill_conditioned"], final["ill_conditioned"]
    assert not final["order_sensitive"], final["order_sensitive"]


def test_thin_truncation_starves_the_tracker_like_the_oracle(gpu):
    """mu = 2 cm in a 128^3 volume over 1.5 m is 1.7 voxels: the first
    frame's band of valid trilinear samples is thinner than the ray-cast's
    coarse step (0.9 mu), so the model maps cover a few percent of the image
    (the oracle's and the GPU's alike), and ICP works from too few
    correspondences - where the benchmark's sessions lost track.  With the
    benchmark's rule, mu = 5 voxels, the same frame covers most of the
    object.  The tracked flags agree with the oracle's frame for frame either
    way (the poses of such frames are ill-conditioned, so only the flags are
    compared; where the oracle's own flag changes with its summation order -
    an iteration on the coarsest level that diverges in one order and not in
    another - the flag must be one the oracle reaches)."""
    depth, _, thin = bench_case("320x240", 128, 6, 1500, mu=0.02)
    _, _, ruled = bench_case("320x240", 128, 6, 1500)
    cover = {}
    for name, cfg in (("thin", thin), ("ruled", ruled)):
        o = O.Session(O.config_from_vs(cfg))
        o.frame(depth[0])
        with V.Session(cfg) as s:
            s.scan_frame_host(depth[0])
            g = s.maps(0)["model_depth"] > 0
        assert (g == (o.maps(0)["model_depth"] > 0)).mean() > 0.99
        cover[name] = g.mean() / (depth[0] > 0).mean()
    assert cover["thin"] < 0.1 and cover["ruled"] > 0.5, cover
    helpers.reanchored_track_check(depth, thin, 6, expect_tracked=False, compare_poses=False)


def test_stages_equal_fused_frame(gpu):
    """The stage-by-stage run above is the fused per-frame graph the
    benchmark times: same poses and maps bit for bit."""
    depth, _, cfg = bench_case("320x240", 128, 4, 1500)
    with V.Session(cfg) as a, V.Session(cfg) as b:
        for k in range(4):
            a.scan_frame_host(depth[k])
            d = torch.from_numpy(np.ascontiguousarray(depth[k]).view(np.int16)).cuda()
            b.stage_filter(d.data_ptr())
            b.stage_track()
            b.stage_integrate()
            b.stage_raycast()
            b.sync()
            assert np.array_equal(a.pose()[1], b.pose()[1]), k
        for l in range(3):
            assert np.array_equal(a.maps(l)["model_vertex"], b.maps(l)["model_vertex"]), l


def test_vga_512_sequence_against_fp64_oracle(gpu):
    nf = 30
    depth, gt, cfg = bench_case("640x480", 512, nf, 2)
    ref = O.Session(O.config_from_vs(cfg, reduce_mode=3, tsdf_store=0), f64=True)
    ours, theirs = [], []
    with V.Session(cfg) as s:
        for k in range(nf):
            T, tracked = s.scan_frame_host(depth[k])
            assert tracked, k
            ours.append(s.pose()[1])
            assert ref.frame(depth[k]), k
            theirs.append(ref.pose_f64())
    d = np.array([helpers.camera_centre_err(a, b) for a, b in zip(ours, theirs)])
    rms = float(np.sqrt(np.mean(d ** 2)))
    print("VGA 512^3, %d frames: camera-centre RMS %.4f mm, max %.4f mm against the FP64 oracle" %
          (nf, rms * 1e3, d.max() * 1e3))
    assert rms < 1e-3 and d.max() < 1e-3

"""Shared set-up for the parity tests: seeded synthetic scenes, matching
product / oracle configurations, pose error metrics."""
import numpy as np

import oracle_py as O
import vs_scanner as V


def make_case(width=160, height=120, dim=128, size=1.0, frames=4, seed=3, f_ref=285.0, mu=0.03,
              noise=1, dropout_iid=0.01, dropout_blob=0.0, max_depth=0.0, cos_normal=-3.0,
              tsdf_type=V.VS_TSDF_INT16, reduce_mode=V.VS_REDUCE_KAHAN, iters=(10, 5, 4), th_icp=0.01):
    """A synthetic sequence plus equivalent vs_config / or_config (config-1 style
    camera scaled to the image width)."""
    f = f_ref * width / 320.0
    sc = V.synth_config(width, height, fx=f, fy=f, cx=width / 2.0, cy=height / 2.0, n_frames=frames, seed=seed,
                        noise=noise, dropout_iid=dropout_iid, dropout_blob=dropout_blob, max_depth=max_depth)
    depth, gt, centre = V.synth_generate(sc)
    origin, vox = V.cube_around(centre, size, dim)
    cfg = V.default_config(width, height, fx=f, fy=f, cx=width / 2.0, cy=height / 2.0, dim=(dim, dim, dim),
                           origin=origin, voxel_size=vox, mu=mu, th_icp=th_icp, cos_normal=cos_normal,
                           icp_iters=iters, tsdf_type=tsdf_type, reduce_mode=reduce_mode)
    ocfg = O.config_from_vs(cfg)
    return dict(depth=depth, gt=gt, centre=centre, cfg=cfg, ocfg=ocfg)


def rot_err(A, B):
    """rotation angle (rad) of A^T B for 4x4 or 3x3 poses; atan2 of the skew
    and symmetric parts, which stays accurate for tiny angles (arccos of the
    trace does not: a float rotation's own orthogonality error would read as
    ~1e-4 rad)"""
    R = np.asarray(A, np.float64)[:3, :3].T @ np.asarray(B, np.float64)[:3, :3]
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
    return float(np.arctan2(np.linalg.norm(w), (np.trace(R) - 1.0) / 2.0))


def trans_err(A, B):
    return float(np.linalg.norm(np.asarray(A, np.float64)[:3, 3] - np.asarray(B, np.float64)[:3, 3]))


def camera_centre_err(A, B):
    """distance between the camera centres of two global->camera poses"""
    def c(T):
        T = np.asarray(T, np.float64)
        return -T[:3, :3].T @ T[:3, 3]
    return float(np.linalg.norm(c(A) - c(B)))


def q16(t):
    """int16 quantisation of a TSDF array (the product's storage)"""
    return np.clip(np.rint(np.asarray(t, np.float32) * np.float32(32767.0)), -32767, 32767).astype(np.int32)


ONE_INT16_STEP = 1.0 / 32767.0


def assert_tsdf_within_one_step(t, ref):
    """TSDF contract: within one int16 quantisation step of the reference's
    value (float storages; int16 storage compares the quantised codes)"""
    d = np.abs(np.asarray(t, np.float64) - np.asarray(ref, np.float64))
    assert d.size and d.max() <= ONE_INT16_STEP * (1.0 + 1e-6), d.max()


def assert_maps_match(depth, vtx, nrm, img, rdepth, rvtx, rnrm, rimg, what=""):
    """Ray-cast contract: the hit masks agree on >= 99.9 % of the pixels, and
    where both hit, vertices and depth within 1 mm on >= 99.9 % of them; the
    normals and the shaded image follow the surface point (normals within
    1e-2, image within 2 levels, on >= 99.9 %)."""
    depth, rdepth = np.asarray(depth).reshape(-1), np.asarray(rdepth).reshape(-1)
    hit, rhit = depth > 0, rdepth > 0
    assert (hit == rhit).mean() >= 0.999, (what, (hit == rhit).mean())
    both = hit & rhit
    assert both.sum() > 0, what
    v, rv = np.asarray(vtx).reshape(-1, 3)[both], np.asarray(rvtx).reshape(-1, 3)[both]
    assert (np.linalg.norm(v - rv, axis=1) <= 1e-3).mean() >= 0.999, what
    assert (np.abs(depth[both] - rdepth[both]) <= 1e-3).mean() >= 0.999, what
    if nrm is not None:
        n, rn = np.asarray(nrm).reshape(-1, 3)[both], np.asarray(rnrm).reshape(-1, 3)[both]
        assert (np.abs(n - rn).max(axis=1) <= 1e-2).mean() >= 0.999, what
    if img is not None:
        i, ri = np.asarray(img).reshape(-1)[both].astype(int), np.asarray(rimg).reshape(-1)[both].astype(int)
        assert (np.abs(i - ri) <= 2).mean() >= 0.999, what


def reanchored_track_check(depth, cfg, frames, expect_tracked=True, compare_poses=True):
    """Runs `frames` frames stage by stage through a session and hands the
    session's own tracking inputs (model maps of the previous ray-cast,
    filtered input pyramid, input normals, previous pose) to the oracle's
    tracker at every frame: the tracked flag must equal the FP32 or the FP64
    oracle's - or, on a frame whose outcome hangs on the summation order
    (the oracle's flag changes with its reduction order there), one of the
    oracle's flags over its orders; such frames are counted, not compared -
    and where both track, the pose must be within 1e-4 rad and 0.1 mm of the
    FP32 and FP64 oracles' (the per-frame tolerance on identical inputs).  A
    frame whose FP32 and FP64 oracles disagree beyond that tolerance on these
    inputs is ill-conditioned (the 6x6 system amplifies rounding; a one-pixel
    change of the coarsest model map can move the solution by a tenth of a
    radian) and is only counted, not compared.  Returns the largest rotation
    (rad) and translation (m) differences, the frames lost and a dict with
    the final pose, volume, maps, the ill-conditioned and the
    order-sensitive frames."""
    import torch

    ocfg = O.config_from_vs(cfg)
    worst = [0.0, 0.0]
    lost, ill, order_sensitive = [], [], []
    with V.Session(cfg) as s:
        for k in range(frames):
            T_prev, T_prev64, _ = s.pose()
            mv = [s.maps(l)["model_vertex"] for l in range(cfg.levels)]
            mn = [s.maps(l)["model_normal"] for l in range(cfg.levels)]
            d = torch.from_numpy(np.ascontiguousarray(depth[k]).view(np.int16)).cuda()
            s.stage_filter(d.data_ptr())
            s.stage_track()
            T, T64, info = s.pose()
            if k > 0:
                m = [s.maps(l) for l in range(cfg.levels)]
                ind = [x["input_depth"] for x in m]
                inn = [x["input_normal"] for x in m] if cfg.cos_normal > -2.0 else None
                ok32, oT, _ = O.track(ocfg, ind, mv, mn, T_prev, innrm_levels=inn, f64=False)
                ok64, dT, _ = O.track(ocfg, ind, mv, mn, T_prev64, innrm_levels=inn, f64=True)
                if bool(info[0]) not in (ok32, ok64):
                    # an iteration that diverges on the coarsest level in one
                    # summation order and not in another: the flag must be
                    # one the oracle reaches with another of its orders
                    alt = {O.track(O.config_from_vs(cfg, reduce_mode=mode), ind, mv, mn,
                                   T_prev64 if f64 else T_prev, innrm_levels=inn, f64=f64)[0]
                           for mode in range(4) for f64 in (False, True)}
                    assert bool(info[0]) in alt, (k, info[0], ok32, ok64)
                    order_sensitive.append(k)
                if expect_tracked:
                    assert ok32 and ok64, (k, ok32, ok64)
                if not info[0]:
                    lost.append(k)
                    assert np.array_equal(T64, T_prev64), k  # a lost frame leaves the pose
                if compare_poses and info[0] and ok64 and k not in order_sensitive:
                    if rot_err(oT, dT) >= 1e-4 or trans_err(oT, dT) >= 1e-4:
                        ill.append(k)
                    else:
                        for ref in (oT, dT):
                            r, t = rot_err(T64, ref), trans_err(T64, ref)
                            worst[0], worst[1] = max(worst[0], r), max(worst[1], t)
                            assert r < 1e-4 and t < 1e-4, (k, r, t)
            s.stage_integrate()
            s.stage_raycast()
            s.sync()
        final = dict(pose=s.pose()[0], volume=s.volume(), maps=[s.maps(l) for l in range(cfg.levels)],
                     ill_conditioned=ill, order_sensitive=order_sensitive)
    return worst, lost, final

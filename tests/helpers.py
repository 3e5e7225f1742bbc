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

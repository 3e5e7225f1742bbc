"""Regenerates the committed golden fixtures (run from the repository root,
in a checkout that has the reference tree mounted; TEST INFRASTRUCTURE ONLY).

refpin.npz
    SE(3) exponentials and 4x4 inverses computed by the reference's own
    STAC/Util/_yooji_math_inlines.h (d_cme_Compute_Matrix_Exponential,
    d_im_Inverse_Matrix_4x4, d_mmm_Multiply_Matrix_Matrix), compiled from the
    reference tree by oracle/build_oracle.py.  These pin the oracle's pose
    algebra bit for bit.
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


if __name__ == "__main__":
    refpin()
    seq_small()
    print("fixtures written to", OUT)

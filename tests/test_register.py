"""Depth -> colour camera registration (vs_warp_depth_to_color, the
reference's z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates): bit-identical
to the oracle's raster-order z-buffer on a two-camera rig, the uint16 form
equal to the float form, and the identity rig giving the input back."""
import numpy as np
import pytest

import oracle_py as O
import vs_scanner as V

W, H = 320, 240
KD = np.array([285.0, 285.0, 160.0, 120.0], np.float32)
KR = np.array([300.0, 298.0, 163.5, 118.25], np.float32)


def rig():
    """a colour camera 5 cm to the side, turned 3 degrees about y"""
    a = np.deg2rad(3.0)
    T = np.eye(4, dtype=np.float32)
    T[0, 0] = T[2, 2] = np.cos(a)
    T[0, 2], T[2, 0] = np.sin(a), -np.sin(a)
    T[0, 3] = -0.05
    return T


def frames():
    sc = V.synth_config(W, H, fx=285.0, fy=285.0, cx=160.0, cy=120.0, n_frames=2, seed=9, dropout_iid=0.02)
    depth, _, _ = V.synth_generate(sc)
    return depth


def test_oracle_identity_rig_returns_the_input():
    mm = frames()[0]
    d = O.depth_to_m(mm)
    out = O.warp_depth(d, KD, np.eye(4, dtype=np.float32), KD, W, H)
    assert np.array_equal(out, d)


@pytest.mark.gpu
def test_warp_matches_oracle_and_uint16_form(gpu):
    torch = pytest.importorskip("torch")
    T = rig()
    for mm in frames():
        d = O.depth_to_m(mm)
        ref = O.warp_depth(d, KD, T, KR, W, H)
        assert (ref > 0).mean() > 0.8
        din = torch.from_numpy(d).cuda()
        dout = torch.empty((H, W), dtype=torch.float32, device="cuda")
        V.warp_depth_to_color(din.data_ptr(), W, H, KD, T, KR, W, H, dout.data_ptr())
        torch.cuda.synchronize()
        got = dout.cpu().numpy()
        assert np.array_equal(got, ref)
        # uint16 form: the same pixels keep the same depth units
        mmin = torch.from_numpy(mm.view(np.int16)).cuda()
        mout = torch.empty((H, W), dtype=torch.int16, device="cuda")
        V.warp_depth_to_color(mmin.data_ptr(), W, H, KD, T, KR, W, H, mout.data_ptr(), mm_scale=0.001)
        torch.cuda.synchronize()
        mm_out = mout.cpu().numpy().view(np.uint16)
        assert np.array_equal(O.depth_to_m(mm_out), got)

"""The ray-cast's free-space skipping: band flags and their distance field.

A march sample reads TSDF 1 wherever the nearest voxel has weight 0 or value
1, and such samples leave the march unchanged, so the march jumps through
boxes of sub-cubes that hold no "band" voxel (weight > 0, value other than
1).  The flags must be exactly the sub-cubes holding a band voxel after every
writer of the volume (integration of every storage, import, carving), and
the distances exactly the Chebyshev distance transform of the flags,
saturating at 8: a flag missing or a distance too large would skip samples
(the parity tests would see the maps change), one too small only costs
speed.  No reference counterpart: the reference marches every step.
"""
import numpy as np
import pytest

import helpers
import vs_scanner as V

pytestmark = pytest.mark.gpu

SAT = 8


def expected_band(s):
    """band flag per sub-cube from the exported volume, (nb_z, nb_y, nb_x)"""
    t, w = s.volume()
    dx, dy, dz = (s.cfg.dim[k] for k in range(3))
    t = t.reshape(dz // 8, 8, dy // 8, 8, dx // 8, 8)
    w = w.reshape(dz // 8, 8, dy // 8, 8, dx // 8, 8)
    return ((w > 0) & (t != 1.0)).any(axis=(1, 3, 5)).astype(np.uint8)


def chebyshev(band):
    """distance in sub-cubes to the nearest flagged one, saturating at SAT
    (brute force over the window of half-width SAT - 1)"""
    d = np.full(band.shape, SAT, np.int32)
    pts = np.argwhere(band > 0)
    if len(pts) == 0:
        return d.astype(np.uint8)
    idx = np.indices(band.shape).reshape(3, -1).T
    for p in pts:
        c = np.abs(idx - p).max(axis=1).reshape(band.shape)
        np.minimum(d, c, out=d)
    return np.minimum(d, SAT).astype(np.uint8)


def check(s):
    band, dist = s.band()
    want = expected_band(s)
    assert want.sum() > 0
    assert np.array_equal(band, want), (int(band.sum()), int(want.sum()))
    assert np.array_equal(dist, chebyshev(want))


@pytest.mark.parametrize("tsdf_type", [V.VS_TSDF_INT16, V.VS_TSDF_FP16, V.VS_TSDF_FP32])
def test_band_after_integration(gpu, tsdf_type):
    c = helpers.make_case(width=160, height=120, dim=64, size=1.0, frames=4, seed=41, tsdf_type=tsdf_type)
    with V.Session(c["cfg"]) as s:
        for k in range(4):
            s.scan_frame_host(c["depth"][k])
        check(s)


def test_band_after_import_and_carving(gpu):
    c = helpers.make_case(width=160, height=120, dim=64, size=1.0, frames=3, seed=42)
    with V.Session(c["cfg"]) as a, V.Session(c["cfg"]) as b:
        for k in range(3):
            a.scan_frame_host(c["depth"][k])
        t, w = a.volume()
        b.set_volume(t, w)
        b.stage_raycast()
        b.sync()
        check(b)
        # carving: the sub-cubes of the last frame's set that lie wholly in
        # the half x < 32 are reset, and with them their flags
        before = int(a.band()[0].sum())
        valid = np.ones((64, 64, 64), np.uint8)
        valid[:, :, :32] = 0
        assert a.uvv_update_valid_volume(valid) > 0
        a.stage_raycast()
        a.sync()
        check(a)
        assert int(a.band()[0].sum()) < before

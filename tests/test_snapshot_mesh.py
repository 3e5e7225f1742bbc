"""Snapshot / resume (vs_session_save / vs_session_load) and surface
extraction (vs_extract_mesh, vs_save_mesh_ply).

A session saved after some frames and loaded again continues bit-identically
to the session that kept running.  The marching-tetrahedra mesh of the GPU
volume equals the oracle's mesh of the same volume as a set of triangles
(same float operations), and a plane's mesh lies on the plane, facing free
space."""
import os

import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V

FRAMES = 6


def _tri_set(xyz):
    """triangles as a sorted array of rows (order-free comparison)"""
    a = np.ascontiguousarray(xyz.reshape(-1, 9))
    return a[np.lexsort(a.T[::-1])]


# ---- oracle known answer (CPU) --------------------------------------------
def test_oracle_mesh_of_a_plane_lies_on_it_and_faces_free_space():
    c = helpers.make_case(width=80, height=60, dim=32, size=1.0, frames=1, seed=2)
    ocfg = c["ocfg"]
    vol = O.Volume(ocfg)
    X, Y, Z = ocfg.dim[0], ocfg.dim[1], ocfg.dim[2]
    z = np.arange(Z, dtype=np.float32)
    plane = 13.3  # voxel z of the surface; TSDF > 0 in front (smaller z)
    tsdf = np.clip((plane - z) / 3.0, -1, 1).astype(np.float32)
    q = np.rint(tsdf * 32767.0) / 32767.0
    t = np.broadcast_to(q[:, None, None], (Z, Y, X)).astype(np.float32).ravel()
    vol.set(t, np.ones(X * Y * Z, np.uint16))
    xyz, _ = vol.mesh()
    # each cell crossed by the plane: tetrahedra {0,7,2,6} and {0,7,5,1} split 2-2
    # (two triangles), the other four 3-1 (one)
    assert len(xyz) == 8 * (X - 1) * (Y - 1)
    zw = (plane + 0.5) / np.float32(1.0 / ocfg.voxel_size) + ocfg.origin[2]
    assert np.allclose(xyz[..., 2], zw, atol=1e-4)
    n = np.cross(xyz[:, 1] - xyz[:, 0], xyz[:, 2] - xyz[:, 0])
    assert (n[:, 2] < 0).all()  # free space is at smaller z
    # the plane is covered: area = (X - 1) (Y - 1) voxels^2
    area = 0.5 * np.linalg.norm(n, axis=1).sum() / ocfg.voxel_size ** 2
    assert abs(area - (X - 1) * (Y - 1)) < 1e-2 * (X - 1) * (Y - 1)


# ---- GPU -------------------------------------------------------------------
@pytest.fixture(scope="module")
def case(gpu):
    return helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=FRAMES, seed=41,
                             cos_normal=float(np.cos(np.deg2rad(20.0))))


@pytest.mark.gpu
def test_mesh_matches_oracle(gpu, case):
    torch = pytest.importorskip("torch")
    vol = O.Volume(case["ocfg"])
    with V.Session(case["cfg"]) as s:
        for k in range(3):
            raw = O.depth_to_m(case["depth"][k])
            Tgc = case["gt"][k].astype(np.float32)
            Tcg = O.pose_inverse(Tgc)
            vol.integrate(raw, Tgc, Tcg)
            d = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (raw, Tgc, Tcg)]
            s.cdtoc_convert_depth_to_tsdf(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr())
        # the extraction compared on the identical volume (integration parity
        # is within one int16 step, tested on its own)
        t, w = vol.get()
        s.set_volume(t, w)
        gxyz, _ = s.mesh()
    oxyz, _ = vol.mesh()
    assert len(oxyz) > 1000
    assert len(gxyz) == len(oxyz)
    assert np.array_equal(_tri_set(gxyz), _tri_set(oxyz))


@pytest.mark.gpu
def test_snapshot_resume_continues_bit_identically(gpu, case, tmp_path):
    path = str(tmp_path / "scan.vssnap")
    with V.Session(case["cfg"]) as a:
        for k in range(3):
            a.scan_frame_host(case["depth"][k])
        a.save(path)
        for k in range(3, FRAMES):
            a.scan_frame_host(case["depth"][k])
        T_a, Td_a, info_a = a.pose()
        t_a, w_a = a.volume()
        m_a = a.maps(0)
    b = V.Session.load(path)
    try:
        assert b.cfg.width == case["cfg"].width and b.cfg.dim[0] == case["cfg"].dim[0]
        for k in range(3, FRAMES):
            b.scan_frame_host(case["depth"][k])
        T_b, Td_b, info_b = b.pose()
        assert np.array_equal(Td_a, Td_b)
        assert np.array_equal(info_a, info_b)
        t_b, w_b = b.volume()
        assert np.array_equal(w_a, w_b) and np.array_equal(t_a, t_b)
        m_b = b.maps(0)
        for k in ("model_depth", "model_vertex", "model_normal"):
            assert np.array_equal(m_a[k], m_b[k]), k
    finally:
        b.close()
    # only sub-cubes with data are stored
    nbr = (case["cfg"].dim[0] // 8) ** 3
    assert os.path.getsize(path) < nbr * 512 * 4 // 2


@pytest.mark.gpu
def test_colour_snapshot_and_coloured_ply(gpu, tmp_path):
    import test_color

    cc = test_color.color_case(frames=3)
    path = str(tmp_path / "c.vssnap")
    with V.Session(cc["cfg"]) as a:
        for k in range(3):
            a.set_color_frame(cc["rgb"][k])
            a.scan_frame_host(cc["depth"][k])
        a.save(path)
        col_a = a.color_volume()
        xyz, rgb = a.mesh(with_color=True)
        ply = str(tmp_path / "m.ply")
        a.save_mesh_ply(ply)
    b = V.Session.load(path)
    try:
        assert np.array_equal(b.color_volume(), col_a)
        xyz_b, rgb_b = b.mesh(with_color=True)
        assert np.array_equal(_tri_set(xyz), _tri_set(xyz_b))
    finally:
        b.close()
    assert len(xyz) > 1000 and (rgb > 0).mean() > 0.9
    with open(ply, "rb") as f:
        head = f.read(512).split(b"end_header\n")[0].decode()
    assert "element vertex %d" % (3 * len(xyz)) in head and "element face %d" % len(xyz) in head
    assert "property uchar red" in head
    size = os.path.getsize(ply)
    assert size == len(head) + len("end_header\n") + 3 * len(xyz) * 15 + len(xyz) * 13


@pytest.mark.gpu
def test_snapshot_rejects_foreign_files(gpu, tmp_path):
    p = tmp_path / "junk.bin"
    p.write_bytes(b"not a snapshot at all" * 10)
    with pytest.raises(V.VsError) as e:
        V.Session.load(str(p))
    assert e.value.code == V.VS_ERR_ARG

"""vs_integrate_depth_noalloc: integration for callers that cannot allocate.

Callers that run inside a host framework's own device-memory pool, real-time
loops that cannot take an allocation's driver lock, or processes that size
all device memory up front cannot use vs_session_create (it allocates the
volume and its scratch).  They own the volume buffer and call the
allocation-free entry point, whose only scratch is a fixed array inside the
library.  Here it is called through the C ABI, twice in a row, and each
result is checked against the session entry point vs_integrate_depth on the
same inputs, with the tolerance of the other parity tests (weights bit-exact,
TSDF within one int16 step).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import helpers
import oracle_py as O
import vs_scanner as V

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def bricked_to_linear(words, dim):
    """bricked int16 + uint16 words -> x-fastest (tsdf q, weight) arrays"""
    nx, ny, nz = dim[0] // 8, dim[1] // 8, dim[2] // 8
    a = np.asarray(words, np.uint32).reshape(nz, ny, nx, 8, 8, 8)  # brick z, y, x; voxel z, y, x
    a = a.transpose(0, 3, 1, 4, 2, 5).reshape(-1)
    q = (a & 0xFFFF).astype(np.uint16).view(np.int16).astype(np.int32)
    w = (a >> 16).astype(np.uint16)
    return q, w


def _host_args(cfg):
    dim = np.array(list(cfg.dim), np.int32)
    origin = np.array(list(cfg.origin), np.float32)
    K = np.array([cfg.fx, cfg.fy, cfg.cx, cfg.cy], np.float32)
    return dim, origin, K


def _compare_two_calls(case):
    """two integrations, each through the session entry point and through the
    allocation-free one, compared after each call"""
    cfg = case["cfg"]
    lib = V.load()
    dim, origin, K = _host_args(cfg)
    nbr = (cfg.dim[0] // 8) * (cfg.dim[1] // 8) * (cfg.dim[2] // 8)
    vol = torch.full((nbr * 512,), 0x7FFF, dtype=torch.int32, device="cuda")  # TSDF 1, weight 0
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    with V.Session(cfg) as s:
        for k in range(2):
            raw = O.depth_to_m(case["depth"][k])
            Tgc = case["gt"][k].astype(np.float32)
            Tcg = O.pose_inverse(Tgc)
            d_raw = torch.from_numpy(raw).cuda()
            d_gc = torch.from_numpy(Tgc).cuda()
            d_cg = torch.from_numpy(Tcg).cuda()
            s.cdtoc_convert_depth_to_tsdf(d_raw.data_ptr(), d_gc.data_ptr(), d_cg.data_ptr())
            rc = lib.vs_integrate_depth_noalloc(ctypes.c_void_p(vol.data_ptr()), p(dim), p(origin),
                                                cfg.voxel_size, cfg.mu, cfg.max_w, ctypes.c_void_p(d_raw.data_ptr()),
                                                cfg.width, cfg.height, p(K), ctypes.c_void_p(d_gc.data_ptr()),
                                                ctypes.c_void_p(d_cg.data_ptr()), None)
            assert rc == V.VS_OK, lib.vs_last_error().decode()
            torch.cuda.synchronize()
            t_ref, w_ref = s.volume()
            q, w = bricked_to_linear(vol.cpu().numpy().view(np.uint32), cfg.dim)
            assert np.array_equal(w, w_ref), k
            m = w_ref > 0
            assert m.sum() > 10000
            assert np.max(np.abs(q[m] - helpers.q16(t_ref[m]))) <= 1, k


def test_noalloc_matches_session_entry_point_on_two_calls(gpu):
    _compare_two_calls(helpers.make_case(width=160, height=120, dim=128, frames=2, seed=3))


def test_noalloc_non_cubic_volume_maps_sub_cubes_like_the_session(gpu):
    case = helpers.make_case(width=160, height=120, dim=128, frames=2, seed=3)
    cfg = case["cfg"]
    # 64 x 128 x 96 voxels around the same scene: sub-cube indices differ per axis
    cfg.dim[0], cfg.dim[1], cfg.dim[2] = 64, 128, 96
    for k in range(3):
        cfg.origin[k] = float(case["centre"][k]) - 0.5 * cfg.dim[k] * cfg.voxel_size
    _compare_two_calls(case)


def test_noalloc_accepts_a_volume_at_its_cap(gpu):
    """512^3 voxels (262,144 sub-cubes, the scratch's maximum) is accepted and
    integrates like the session entry point"""
    case = helpers.make_case(width=160, height=120, dim=512, size=1.0, frames=2, seed=3)
    _compare_two_calls(case)


def test_noalloc_rejects_volumes_beyond_its_scratch(gpu):
    lib = V.load()
    dim = np.array([1024, 1024, 1024], np.int32)  # 2,097,152 sub-cubes > 262,144
    origin = np.zeros(3, np.float32)
    K = np.array([525.0, 525.0, 319.5, 239.5], np.float32)
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    ptr = ctypes.c_void_p(buf.data_ptr())
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = lib.vs_integrate_depth_noalloc(ptr, p(dim), p(origin), 0.001, 0.02, 100.0, ptr, 640, 480, p(K), ptr, ptr,
                                        None)
    assert rc == V.VS_ERR_ARG
    assert b"at most 262144" in lib.vs_last_error()

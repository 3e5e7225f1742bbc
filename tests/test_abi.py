"""The C-ABI library: it loads, exports every symbol include/vs.h declares,
and rejects bad input on the host.  No compute call is made here (these tests
run without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import vs_scanner as V

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "vs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vs_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(V.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(built):
    assert set(declared_symbols()) == set(V._SIGS)


def test_library_links_cuda_runtime_not_a_fallback(built):
    # the product has no CPU path: the library depends on the CUDA runtime
    import subprocess
    out = subprocess.run(["ldd", V.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcudart" in out


def _cfg(**kw):
    args = dict(dim=(512, 512, 512), voxel_size=1.5 / 512)
    args.update(kw)
    return V.default_config(640, 480, **args)


def test_session_bytes_config_two(built):
    b = V.load().vs_session_bytes(ctypes.byref(_cfg()))
    assert 512 * 1024 ** 2 < b < 640 * 1024 ** 2  # int16 + uint16 pairs: 4 bytes per voxel


@pytest.mark.parametrize("field,value", [("levels", 0), ("levels", 4), ("width", 4), ("width", 4096),
                                         ("voxel_size", 0.0), ("mu", -1.0), ("max_w", 0.0), ("th_icp", 0.0),
                                         ("tsdf_type", 7), ("reduce_mode", 3)])
def test_invalid_config_rejected_before_any_device_work(built, field, value):
    c = _cfg()
    setattr(c, field, value)
    assert V.load().vs_session_bytes(ctypes.byref(c)) == 0
    h = ctypes.c_void_p()
    assert V.load().vs_session_create(ctypes.byref(c), ctypes.byref(h)) == V.VS_ERR_ARG
    assert V.load().vs_last_error()


def test_invalid_dims_rejected(built):
    c = _cfg(dim=(500, 512, 512))
    h = ctypes.c_void_p()
    assert V.load().vs_session_create(ctypes.byref(c), ctypes.byref(h)) == V.VS_ERR_ARG


def test_null_arguments_rejected(built):
    lib = V.load()
    assert lib.vs_session_create(None, None) == V.VS_ERR_ARG
    assert lib.vs_scan_frame(None, None, None) == V.VS_ERR_ARG
    assert lib.vs_track_pose(None, None, None) == V.VS_ERR_ARG
    assert lib.vs_get_pose(None, None, None, None) == V.VS_ERR_ARG
    assert lib.vs_get_band(None, None, None) == V.VS_ERR_ARG
    assert lib.vs_get_icp_system(None, None, None) == V.VS_ERR_ARG
    assert lib.vs_batch_step(None, None, 0, None, None) == V.VS_ERR_ARG
    assert lib.vs_batch_step_host(None, None, 0, None, None, None) == V.VS_ERR_ARG


def test_no_gpu_means_error_not_fallback(built):
    if V.device_count() > 0:
        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    rc = V.load().vs_session_create(ctypes.byref(_cfg()), ctypes.byref(h))
    assert rc == V.VS_ERR_CUDA


def test_noalloc_rejects_a_misaligned_volume_before_any_launch(built):
    """the allocation-free entry point checks the caller's volume pointer
    (16-byte aligned) before it touches the GPU, so the call fails the same
    way with or without a device"""
    import vs_scanner as V

    lib = V.load()
    dim = np.array([64, 64, 64], np.int32)
    origin = np.zeros(3, np.float32)
    K = np.array([525.0, 525.0, 319.5, 239.5], np.float32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    fake = ctypes.c_void_p(0x10008)  # 8-byte aligned only; never dereferenced
    rc = lib.vs_integrate_depth_noalloc(fake, p(dim), p(origin), 0.005, 0.02, 100.0, fake, 640, 480, p(K), fake,
                                        fake, None)
    assert rc == V.VS_ERR_ARG
    assert b"16-byte aligned" in lib.vs_last_error()

"""bench.py's measurement helpers on the CPU: the pose the precision study
hands the oracle, the per-unit figures its roofline scales, and the unit
counts of a step."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import vs_scanner as V  # noqa: E402


def _rigid(rng):
    a = rng.normal(size=3)
    a *= rng.uniform(0.1, 3.0) / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    th = np.linalg.norm(a)
    R = np.eye(3) + np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = rng.uniform(-2, 2, size=3)
    return T


def test_device_inverse_is_the_rigid_inverse():
    rng = np.random.default_rng(3)
    for _ in range(20):
        T = _rigid(rng)
        Ti = bench._device_inverse(T)
        assert Ti.dtype == np.float32
        assert np.allclose(Ti.astype(np.float64), np.linalg.inv(T), atol=1e-6)
        # the float rounding of the FP64 inverse, element for element
        assert np.array_equal(Ti[:3, :3], T[:3, :3].T.astype(np.float32))


def test_per_unit_figures_come_from_the_committed_profiles():
    for key in ("dram_bytes", "warp_inst"):
        pu = bench.raycast_per_unit(key)
        assert pu is not None and pu[0] > 0 and pu[1] > 0, key
    assert bench.traffic_per_unit("k_icp_iter", "dram_bytes_per_pixel") > 0
    assert bench.traffic_per_unit("k_integrate", "dram_bytes_per_voxel") > 0
    assert bench.traffic_per_unit("no_such_kernel", "dram_bytes_per_ray") is None


def test_unit_counts_of_a_session():
    cfg = V.default_config(640, 480, dim=(512, 384, 256))
    assert bench.level_pixels(cfg) == [640 * 480, 320 * 240, 160 * 120]
    assert bench.level_bricks(cfg) == 64 * 48 * 32

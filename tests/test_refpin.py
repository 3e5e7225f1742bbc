"""The oracle's pose algebra against the reference's own host math.

STAC/Util/_yooji_math_inlines.h builds on Linux from the reference tree; its
outputs on fixed inputs are committed in tests/golden/refpin.npz (written by
tests/golden/gen_golden.py), and where the tree is mounted the harness is also
rebuilt and compared live."""
import ctypes
import os

import numpy as np
import pytest

import oracle_py as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin.npz")


def test_se3_exp_matches_reference_bit_for_bit(built):
    g = np.load(GOLD)
    for xi, e in zip(g["xi"], g["exp"]):
        assert np.array_equal(O.se3_exp(xi).reshape(16), e)


def test_inverse4_matches_reference_bit_for_bit(built):
    g = np.load(GOLD)
    for m, inv in zip(g["mats"], g["inv"]):
        assert np.array_equal(O.pose_inverse(m).reshape(16), inv)


def test_fp64_exp_agrees_with_reference_to_float_precision(built):
    g = np.load(GOLD)
    for xi, e in zip(g["xi"], g["exp"]):
        d = O.se3_exp(xi.astype(np.float64), f64=True).reshape(16)
        assert np.max(np.abs(d - e.astype(np.float64))) < 2e-6


def test_live_reference_harness(built):
    ref = O.load_ref_pin()
    if ref is None:
        pytest.skip("reference tree not mounted on this host")
    rng = np.random.default_rng(5)
    for _ in range(200):
        xi = (rng.standard_normal(6) * 10.0 ** rng.uniform(-5, -0.5)).astype(np.float32)
        e = np.empty(16, np.float32)
        ref.ref_se3_exp(xi.ctypes.data_as(ctypes.c_void_p), e.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(O.se3_exp(xi).reshape(16), e)
        m = e.copy()
        m[3], m[7], m[11] = rng.uniform(-1, 1, 3).astype(np.float32)
        inv = np.empty(16, np.float32)
        ref.ref_inverse4(m.ctypes.data_as(ctypes.c_void_p), inv.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(O.pose_inverse(m).reshape(16), inv)

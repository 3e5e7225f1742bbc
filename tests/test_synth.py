"""The seeded synthetic sequence generator (host code)."""
import numpy as np

import vs_scanner as V


def test_deterministic_and_seeded(built):
    a = V.synth_generate(V.synth_config(64, 48, n_frames=3, seed=4))
    b = V.synth_generate(V.synth_config(64, 48, n_frames=3, seed=4, threads=1))
    c = V.synth_generate(V.synth_config(64, 48, n_frames=3, seed=5))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])


def test_first_pose_is_identity_and_poses_are_rigid(built):
    d, T, c = V.synth_generate(V.synth_config(64, 48, n_frames=20, seed=2))
    assert np.allclose(T[0], np.eye(4), atol=1e-12)
    for M in T:
        assert np.allclose(M[:3, :3] @ M[:3, :3].T, np.eye(3), atol=1e-12)
        assert np.allclose(M[3], [0, 0, 0, 1])
    # orbit: the camera centre stays ~1 m from the scene centre
    for M in T:
        C = -M[:3, :3].T @ M[:3, 3]
        assert abs(np.linalg.norm(C - c) - 1.0) < 0.01


def test_dropout_and_cutoff(built):
    d, _, _ = V.synth_generate(V.synth_config(320, 240, fx=285, fy=285, cx=160, cy=120, n_frames=1, seed=1,
                                              noise=0))
    base = (d[0] == 0).mean()
    d2, _, _ = V.synth_generate(V.synth_config(320, 240, fx=285, fy=285, cx=160, cy=120, n_frames=1, seed=1,
                                               noise=0, dropout_iid=0.01))
    assert 0.007 < (d2[0] == 0).mean() - base < 0.013
    d3, _, _ = V.synth_generate(V.synth_config(640, 480, n_frames=1, seed=1, dropout_blob=0.015, max_depth=2.5))
    assert d3[0].max() <= 2500
    assert (d3[0] == 0).mean() > 0.01


def test_axial_noise_scale(built):
    cfg = dict(n_frames=1, seed=3, jitter_deg=0.0, jitter_m=0.0)
    clean, _, _ = V.synth_generate(V.synth_config(320, 240, noise=0, **cfg))
    noisy, _, _ = V.synth_generate(V.synth_config(320, 240, noise=1, **cfg))
    m = (clean[0] > 0) & (noisy[0] > 0) & (clean[0] < 1500)
    diff = noisy[0][m].astype(np.float64) - clean[0][m]
    z = clean[0][m] / 1000.0
    sig = (0.0012 + 0.0019 * (z - 0.4) ** 2) * 1000.0
    ratio = np.std(diff / np.sqrt(sig ** 2 + 1.0 / 6.0))  # quantisation of both maps adds ~1/6 mm^2
    assert 0.85 < ratio < 1.15

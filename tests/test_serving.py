"""Serving loop (vs_server_*): continuous batching, admission by HBM budget,
and each session's results the same alone and in the mix.

Frames of several sessions are submitted in a seeded random interleaving with
bursts and pauses, so the steps that carry them have varying membership and
size; every per-frame pose the server returns, and every session's final
volume, must equal those of the session run alone (bit-identical: the batch
kernels keep each session's work and summation order)."""
import time

import numpy as np
import pytest

import helpers
import vs_scanner as V

pytestmark = pytest.mark.gpu

FRAMES = 6


def _cases():
    a = helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=FRAMES, seed=21)
    b = helpers.make_case(width=320, height=240, dim=128, size=1.0, frames=FRAMES, seed=22,
                          cos_normal=float(np.cos(np.deg2rad(20.0))))
    c = helpers.make_case(width=256, height=212, dim=64, size=1.0, frames=FRAMES, seed=23)
    d = helpers.make_case(width=160, height=120, dim=128, size=1.0, frames=FRAMES, seed=24, iters=(6, 3, 3))
    return [a, b, c, d]


@pytest.fixture(scope="module")
def cases(gpu):
    return _cases()


@pytest.fixture(scope="module")
def alone(cases):
    out = []
    for c in cases:
        with V.Session(c["cfg"]) as s:
            poses = [s.scan_frame_host(c["depth"][k])[0].copy() for k in range(FRAMES)]
            t, w = s.volume()
            out.append(dict(poses=poses, tsdf=t, w=w))
    return out


def _collect(srv, want, timeout_s=60.0):
    got = []
    t0 = time.time()
    while len(got) < want and time.time() - t0 < timeout_s:
        got += srv.poll(timeout_ms=200)
    return got


@pytest.mark.parametrize("lanes,pipeline", [(1, 2), (2, 1), (3, 2)])
def test_serving_equals_alone_in_a_random_mix(cases, alone, lanes, pipeline):
    """one lane, or several lanes whose steps run at the same time on their
    own streams: the same per-frame poses and final volumes"""
    rng = np.random.default_rng(5)
    with V.Server(lanes=lanes, pipeline=pipeline) as srv:
        ids = [srv.open(c["cfg"]) for c in cases]
        assert all(srv.state(i) == V.VS_SESSION_RESIDENT for i in ids)
        order = [i for i in range(len(cases)) for _ in range(FRAMES)]
        rng.shuffle(order)
        nxt = [0] * len(cases)
        for j, i in enumerate(order):
            while not srv.submit(ids[i], cases[i]["depth"][nxt[i]]):
                time.sleep(0.001)
            nxt[i] += 1
            if rng.random() < 0.3:
                time.sleep(float(rng.uniform(0.0, 0.004)))
        res = _collect(srv, len(order))
        srv.drain()
        assert len(res) == len(order)
        st = srv.stats()
        assert st["frames"] == len(order)
        for r in res:
            i = ids.index(r["session"])
            assert np.array_equal(r["T_gc"], alone[i]["poses"][r["frame"]]), (i, r["frame"])
            assert r["latency_ms"] > 0
            assert 1 <= r["batch"] <= len(cases)
        # per session the frames come back in order
        for sid in ids:
            fr = [r["frame"] for r in res if r["session"] == sid]
            assert fr == list(range(FRAMES))
        for i, sid in enumerate(ids):
            t, w = srv.session(sid).volume()
            assert np.array_equal(w, alone[i]["w"]), i
            assert np.array_equal(t, alone[i]["tsdf"]), i


def test_admission_waits_for_budget(cases, alone):
    cfg = cases[0]["cfg"]
    need = V.load().vs_session_bytes(cfg)
    # room for two sessions of this config, not three
    with V.Server(hbm_budget=2 * need + need // 2) as srv:
        a = srv.open(cfg)
        b = srv.open(cfg)
        c = srv.open(cfg)
        assert srv.state(a) == V.VS_SESSION_RESIDENT
        assert srv.state(b) == V.VS_SESSION_RESIDENT
        assert srv.state(c) == V.VS_SESSION_WAITING
        for k in range(3):
            assert srv.submit(c, cases[0]["depth"][k])   # queued while waiting
            assert srv.submit(a, cases[0]["depth"][k])
        res = _collect(srv, 3)
        assert {r["session"] for r in res} == {a}
        st = srv.stats()
        assert st["resident"] == 2 and st["waiting"] == 1
        srv.close_session(a)  # frees its memory: c is admitted and runs its queued frames
        res2 = _collect(srv, 3)
        srv.drain()
        assert srv.state(c) == V.VS_SESSION_RESIDENT
        assert srv.state(a) == V.VS_SESSION_CLOSED
        assert [r["frame"] for r in res2 if r["session"] == c] == [0, 1, 2]
        for r in res2:
            assert np.array_equal(r["T_gc"], alone[0]["poses"][r["frame"]])
        for r in res:
            assert np.array_equal(r["T_gc"], alone[0]["poses"][r["frame"]])
        # c waited for admission, so its first frame's latency covers the wait
        assert max(r["latency_ms"] for r in res2) > 0


def test_server_argument_errors(cases):
    cfg = cases[0]["cfg"]
    need = V.load().vs_session_bytes(cfg)
    with V.Server(hbm_budget=need + 1, queue_depth=2) as srv:
        a = srv.open(cfg)
        b = srv.open(cfg)  # waits: the budget holds one
        assert srv.state(b) == V.VS_SESSION_WAITING
        assert srv.submit(b, cases[0]["depth"][0])
        assert srv.submit(b, cases[0]["depth"][1])
        assert not srv.submit(b, cases[0]["depth"][2])  # queue_depth frames already wait
        with pytest.raises(V.VsError) as e:
            srv.submit(12345, cases[0]["depth"][0])
        assert e.value.code == V.VS_ERR_ARG
        big = V.default_config(cfg.width, cfg.height)
        for f, _ in V.VsConfig._fields_:
            setattr(big, f, getattr(cfg, f))
        big.dim[0] = big.dim[1] = big.dim[2] = 512
        with pytest.raises(V.VsError) as e:
            srv.open(big)
        assert e.value.code == V.VS_ERR_MEMORY
        srv.close_session(b)
        assert srv.state(b) == V.VS_SESSION_CLOSED
        with pytest.raises(V.VsError) as e:
            srv.submit(b, cases[0]["depth"][0])
        assert e.value.code == V.VS_ERR_STATE
        srv.close_session(a)

"""Batched frames (vs_batch_*): each session's results are the same alone and
in a batch.

Sessions of different frame sizes, volumes, pyramid depths, iteration counts
and normal-test settings are advanced once through their own per-frame graph
(vs_scan_frame_host) and once through batch steps whose membership changes
from step to step.  The FP64 master pose, the float pose, the frame result,
the whole TSDF volume and every level's model maps must be bit-identical: a
session's work items and summation order do not depend on what else shares a
launch, so the tolerance here is zero."""
import numpy as np
import pytest

import helpers
import vs_scanner as V

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FRAMES = 5


def _cases():
    a = helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=FRAMES, seed=11,
                          cos_normal=float(np.cos(np.deg2rad(20.0))))
    b = helpers.make_case(width=320, height=240, dim=128, size=1.0, frames=FRAMES, seed=5, dropout_blob=0.01)
    c = helpers.make_case(width=256, height=212, dim=64, size=1.0, frames=FRAMES, seed=7, iters=(8, 4, 2))
    c["cfg"].levels = 2
    return [a, b, c]


def _snapshot(s):
    T, Td, info = s.pose()
    t, w = s.volume()
    maps = [s.maps(l) for l in range(s.cfg.levels)]
    return dict(T=T, Td=Td, info=info, tsdf=t, w=w, maps=maps)


def _assert_same(a, b, tag):
    assert np.array_equal(a["Td"], b["Td"]), tag
    assert np.array_equal(a["T"], b["T"]), tag
    assert np.array_equal(a["info"], b["info"]), tag
    assert np.array_equal(a["w"], b["w"]), tag
    assert np.array_equal(a["tsdf"], b["tsdf"]), tag
    for l, (ma, mb) in enumerate(zip(a["maps"], b["maps"])):
        for k in ("model_depth", "model_vertex", "model_normal", "model_img", "input_depth"):
            assert np.array_equal(ma[k], mb[k]), (tag, l, k)


@pytest.fixture(scope="module")
def cases(gpu):
    return _cases()


@pytest.fixture(scope="module")
def alone(cases):
    out = []
    for c in cases:
        with V.Session(c["cfg"]) as s:
            snaps = []
            for k in range(FRAMES):
                s.scan_frame_host(c["depth"][k])
                snaps.append(_snapshot(s))
            out.append(snaps)
    return out


# which sessions take a frame at each step; every session gets FRAMES frames
SCHEDULE = [[0, 1, 2], [0, 2], [1], [0, 1, 2], [2, 0], [1, 0], [1, 2], [0, 1, 2]]


def test_batch_equals_alone_with_changing_membership(cases, alone):
    sessions = [V.Session(c["cfg"]) for c in cases]
    done = [0, 0, 0]
    try:
        with V.Batch() as b:
            kernels = set()
            for step in SCHEDULE:
                members = [i for i in step if done[i] < FRAMES]
                if not members:
                    continue
                frames = [cases[i]["depth"][done[i]] for i in members]
                T, tracked = b.step_host([sessions[i] for i in members], frames)
                kernels.add(b.kernels_per_step())
                for j, i in enumerate(members):
                    snap = _snapshot(sessions[i])
                    _assert_same(snap, alone[i][done[i]], "session %d frame %d" % (i, done[i]))
                    assert np.array_equal(T[j], snap["T"])
                    assert bool(tracked[j]) == bool(snap["info"][0])
                    done[i] += 1
            assert done == [FRAMES] * 3
            # one graph for every membership: the launch count does not depend on the batch size
            assert len(kernels) == 1
    finally:
        for s in sessions:
            s.close()


def test_batch_device_frames_and_async_step(cases, alone):
    sessions = [V.Session(c["cfg"]) for c in cases]
    try:
        with V.Batch() as b:
            for k in range(2):
                frames = [torch.from_numpy(c["depth"][k].view(np.int16)).cuda() for c in cases]
                torch.cuda.synchronize()
                b.step(sessions, [f.data_ptr() for f in frames])
                b.sync()
                for i, s in enumerate(sessions):
                    _assert_same(_snapshot(s), alone[i][k], "device frames, session %d frame %d" % (i, k))
    finally:
        for s in sessions:
            s.close()


def test_batch_pinned_host_frames_read_in_place(cases, alone):
    """pinned host frames are read by the step's first kernel over the host
    link, pageable ones copied first: the same results either way"""
    sessions = [V.Session(c["cfg"]) for c in cases]
    try:
        with V.Batch() as b:
            for k in range(2):
                pinned = [torch.from_numpy(c["depth"][k].view(np.int16)).pin_memory() for c in cases]
                frames = [p.numpy().view(np.uint16) for p in pinned]
                if k == 1:
                    frames[1] = np.array(cases[1]["depth"][k])  # one pageable frame in the mix
                b.step_host(sessions, frames)
                for i, s in enumerate(sessions):
                    _assert_same(_snapshot(s), alone[i][k], "pinned frames, session %d frame %d" % (i, k))
    finally:
        for s in sessions:
            s.close()


def test_full_batch_of_small_sessions(gpu):
    """VS_MAX_BATCH sessions in one step; a few are checked against their run alone"""
    case = helpers.make_case(width=64, height=48, dim=32, size=1.0, frames=2, seed=13)
    cfgs = []
    for i in range(V.VS_MAX_BATCH):
        c = V.default_config(64, 48)
        ctypes_copy = case["cfg"]
        for f, _ in V.VsConfig._fields_:
            setattr(c, f, getattr(ctypes_copy, f))
        c.dim[0] = c.dim[1] = c.dim[2] = 32 + 8 * (i % 3)
        c.voxel_size = 1.0 / c.dim[0]
        cfgs.append(c)
    sessions = [V.Session(c) for c in cfgs]
    try:
        with V.Batch() as b:
            for k in range(2):
                b.step_host(sessions, [case["depth"][k]] * len(sessions))
            for i in (0, 1, 2, 63):
                with V.Session(cfgs[i]) as s:
                    for k in range(2):
                        s.scan_frame_host(case["depth"][k])
                    _assert_same(_snapshot(sessions[i]), _snapshot(s), "slot %d" % i)
    finally:
        for s in sessions:
            s.close()


def test_batch_argument_errors(cases):
    a = V.Session(cases[0]["cfg"])
    cfg = cases[1]["cfg"]
    other = V.default_config(cfg.width, cfg.height)
    for f, _ in V.VsConfig._fields_:
        setattr(other, f, getattr(cfg, f))
    other.tsdf_type = V.VS_TSDF_FP32
    b2 = V.Session(other)
    frame = cases[0]["depth"][0]
    try:
        with V.Batch() as b:
            with pytest.raises(V.VsError) as e:
                b.step_host([a, a], [frame, frame])
            assert e.value.code == V.VS_ERR_ARG
            with pytest.raises(V.VsError) as e:
                b.step_host([a, b2], [frame, cases[1]["depth"][0]])
            assert e.value.code == V.VS_ERR_ARG
            with pytest.raises(V.VsError) as e:
                b.step_host([], [])
            assert e.value.code == V.VS_ERR_ARG
            with pytest.raises(V.VsError) as e:
                b.step_host([a] * (V.VS_MAX_BATCH + 1), [frame] * (V.VS_MAX_BATCH + 1))
            assert e.value.code == V.VS_ERR_ARG
    finally:
        a.close()
        b2.close()

"""Launch-shape autotuner of the batch runner (vs_batch_autotune).

A launch shape (how a warp's 32 rays are tiled, how many blocks per SM the
ray-cast grids hold, the rows of the filter / activation tile, the update
grid of the integration) changes only time: every shape must give
bit-identical poses, volumes and maps, the tuner must leave every session's
state as it was (it re-runs the ray-cast and the filter on the current data
and the integration as a dry run), and a tuned runner must continue the
sequence exactly as an untuned one."""
import numpy as np
import pytest

import helpers
import vs_scanner as V

pytestmark = pytest.mark.gpu

FRAMES = 4


def _snapshot(s):
    T, Td, info = s.pose()
    t, w = s.volume()
    return dict(Td=Td, info=info, tsdf=t, w=w, maps=[s.maps(l) for l in range(s.cfg.levels)])


def _same(a, b, tag):
    assert np.array_equal(a["Td"], b["Td"]), tag
    assert np.array_equal(a["info"], b["info"]), tag
    assert np.array_equal(a["w"], b["w"]), tag
    assert np.array_equal(a["tsdf"], b["tsdf"]), tag
    for l, (ma, mb) in enumerate(zip(a["maps"], b["maps"])):
        for k in ("model_depth", "model_vertex", "model_normal", "model_img", "input_depth"):
            assert np.array_equal(ma[k], mb[k]), (tag, l, k)


@pytest.fixture(scope="module")
def cases(gpu):
    return [helpers.make_case(width=160, height=120, dim=96, size=0.75, frames=FRAMES, seed=31),
            helpers.make_case(width=320, height=240, dim=128, size=1.0, frames=FRAMES, seed=32)]


def _run(cases, shape=None, tune_after=None, device_frames=False):
    ss = [V.Session(c["cfg"]) for c in cases]
    snaps = []
    with V.Batch() as b:
        if shape is not None:
            b.set_launch_shape(*shape)
        for k in range(FRAMES):
            if device_frames:
                # frames read in place by the step: the tuner's filter re-run
                # reads the sessions' own copies, kept current by the ingest
                torch = pytest.importorskip("torch")
                fr = [torch.from_numpy(c["depth"][k].view(np.int16)).cuda() for c in cases]
                torch.cuda.synchronize()
                b.step(ss, [f.data_ptr() for f in fr])
                b.sync()
                del fr
            else:
                b.step_host(ss, [c["depth"][k] for c in cases])
            if tune_after == k:
                before = [_snapshot(s) for s in ss]
                best, ms = b.autotune(ss, reps=2)
                assert 1 <= best[0] <= 5 and best[1] >= 1 and ms > 0
                assert best[3] in (4, 8, 16) and best[4] in (0, 2, 3)
                assert b.launch_shape() == best
                for s, snap in zip(ss, before):
                    _same(_snapshot(s), snap, "state after autotune")
        snaps = [_snapshot(s) for s in ss]
    for s in ss:
        s.close()
    return snaps


def test_every_launch_shape_gives_the_same_results(cases):
    ref = _run(cases)
    for shape in [(5, 4, 0), (1, 0, 3), (4, 2, 2), (3, 0, 0, 4, 2), (2, 0, 0, 16, 3)]:
        got = _run(cases, shape=shape)
        for i, (a, b) in enumerate(zip(ref, got)):
            _same(a, b, "shape %s session %d" % (shape, i))


@pytest.mark.parametrize("device_frames", [False, True])
def test_autotune_keeps_state_and_results(cases, device_frames):
    ref = _run(cases)
    got = _run(cases, tune_after=1, device_frames=device_frames)
    for i, (a, b) in enumerate(zip(ref, got)):
        _same(a, b, "tuned session %d" % i)


def test_launch_shape_rejects_out_of_range(cases):
    with V.Batch() as b:
        with pytest.raises(V.VsError) as e:
            b.set_launch_shape(6)
        assert e.value.code == V.VS_ERR_ARG
        assert b.launch_shape()[0] == 3
        for bad in [(3, 0, 0, 5, 0), (3, 0, 0, 8, 33)]:
            with pytest.raises(V.VsError):
                b.set_launch_shape(*bad)

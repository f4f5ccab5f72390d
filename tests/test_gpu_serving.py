"""Serving on the GPU: 8 simulated cameras (4 x 1280x720 @ 60 fps, 4 x
1920x1080 @ 30 fps) with Poisson arrivals go through the continuous-batching
server; every result must equal the result of detecting that frame alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_each_result_is_the_same_alone_and_in_the_mix():
    from atag import serving, synth
    from atag.detector import Detector
    specs = [synth.FrameSpec(1280, 720, 20, (16, 200), 150, (0.5, 1.5), (2.0, 8.0))] * 4 + \
            [synth.FrameSpec(1920, 1080, 40, (16, 300), 300, (0.5, 1.5), (2.0, 8.0))] * 4
    cams = [[synth.render(s, 100 * c + k) for k in range(2)] for c, s in enumerate(specs)]
    # results alone
    alone = {}
    det = Detector(1920, 1080)
    for c, frames in enumerate(cams):
        for k, f in enumerate(frames):
            q, st = det.detect([torch.from_numpy(f).cuda()])
            alone[(c, k)] = q[0]
    slots = serving.executors_for_memory(1920, 1080, 8, 8 * 1920 * 1080, max_slots=3)
    assert len(slots) == 3
    srv = serving.Server(slots)
    rates = [60.0] * 4 + [30.0] * 4
    res = serving.run_cameras(srv, cams, rates, duration_s=1.5, seed=3)
    assert len(res) > 300
    counters = {}
    for r in res:
        k = counters.get(r.camera, 0)
        counters[r.camera] = k + 1
        want = alone[(r.camera, k % 2)]
        assert r.quads.tobytes() == want.tobytes(), (r.seq, r.camera)
        assert int(r.stats["status"]) == 0
    summ = serving.latency_summary(res, 1.5)
    assert summ["p99_ms"] < 100.0
    print(summ)


def _cameras():
    from atag import synth
    specs = [synth.FrameSpec(1280, 720, 20, (16, 200), 150, (0.5, 1.5), (2.0, 8.0))] * 4 + \
            [synth.FrameSpec(1920, 1080, 40, (16, 300), 300, (0.5, 1.5), (2.0, 8.0))] * 4
    return [[synth.render(s, 100 * c + k) for k in range(2)] for c, s in enumerate(specs)]


def _alone(cams):
    from atag.detector import Detector
    det = Detector(1920, 1080)
    out = {}
    for c, frames in enumerate(cams):
        for k, f in enumerate(frames):
            q, st = det.detect([torch.from_numpy(f).cuda()])
            out[(c, k)] = q[0]
    return out


def _check_same_as_alone(res, alone):
    counters = {}
    for r in res:
        k = counters.get(r.camera, 0)
        counters[r.camera] = k + 1
        assert r.quads.tobytes() == alone[(r.camera, k % 2)].tobytes(), (r.seq, r.camera, r.batch_size)
        assert int(r.stats["status"]) == 0


def test_bursts_are_batched_and_slots_overlap():
    """16 requests arriving at once: the first free slot takes as many as
    its budget allows (a batch of several frames), the next slot the rest,
    so two slots are on the GPU together; every result is the frame's
    result detected alone."""
    from atag import serving
    cams = _cameras()
    alone = _alone(cams)
    slots = serving.executors_for_memory(1920, 1080, 8, 8 * 1920 * 1080, max_slots=3)
    srv = serving.Server(slots)
    res = serving.run_bursts(srv, cams, n_bursts=20, burst_size=16, period_s=0.02)
    assert len(res) == 320
    assert srv.max_in_flight >= 2
    assert max(r.batch_size for r in res) > 1
    _check_same_as_alone(res, alone)


def test_overloaded_cameras_are_batched():
    """8 cameras at 16 times the camera rates (4 x 720p @ 960 Hz, 4 x 1080p
    @ 480 Hz: 5,760 requests/s, more than one launch per request can keep
    up with): requests that arrive while the slots are busy are admitted
    together, and the results stay those of each frame alone."""
    from atag import serving
    cams = _cameras()
    alone = _alone(cams)
    # the cameras deliver into pinned capture buffers
    pinned = [[torch.from_numpy(f).pin_memory() for f in fr] for fr in cams]
    slots = serving.executors_for_memory(1920, 1080, 8, 8 * 1920 * 1080, max_slots=3)
    srv = serving.Server(slots)
    serving.warm(srv, pinned[4][0])
    res = serving.run_cameras(srv, pinned, [960.0] * 4 + [480.0] * 4, duration_s=1.0, seed=9)
    assert len(res) > 4000
    assert srv.max_in_flight >= 2
    assert max(r.batch_size for r in res) > 1
    _check_same_as_alone(res, alone)
    print(serving.latency_summary(res, 1.0))

"""CPU tests of the continuous-batching scheduler (atag.serving) with a fake
executor standing in for a GPU slot."""
import numpy as np

from atag import serving


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    """Completes a launch `delay` seconds of fake time later; the result for
    a frame is its pixel sum, so results can be matched to requests."""

    def __init__(self, clock, delay, max_frames=4, max_pixels=10_000):
        self.clock, self.delay = clock, delay
        self.max_frames, self.max_pixels = max_frames, max_pixels
        self.frames, self.t_done, self.launches = None, None, []

    def capacity(self):
        return self.max_frames, self.max_pixels

    def launch(self, frames):
        assert self.frames is None, "launched while busy"
        self.frames = frames
        self.t_done = self.clock() + self.delay
        self.launches.append(len(frames))

    def done(self):
        return self.clock() >= self.t_done

    def results(self):
        out = [(np.array([f.sum()]), np.zeros(1)) for f in self.frames]
        self.frames = None
        return out


def _frame(v, shape=(8, 8)):
    return np.full(shape, v, np.uint8)


def test_every_request_is_served_with_its_own_result():
    clock = FakeClock()
    slots = [FakeExecutor(clock, 0.010) for _ in range(2)]
    srv = serving.Server(slots, clock=clock)
    for i in range(40):
        clock.t = i * 0.001
        srv.submit(serving.Request(i, i % 3, _frame(i), clock.t))
        srv.poll()
    while not srv.idle():
        clock.t += 0.001
        srv.poll()
    res = sorted(srv.completed, key=lambda r: r.seq)
    assert [r.seq for r in res] == list(range(40))
    for r in res:
        assert int(r.quads[0]) == r.seq * 64
        assert r.t_done >= r.t_arrival


def test_requests_arriving_while_busy_are_batched_and_slots_overlap():
    clock = FakeClock()
    slots = [FakeExecutor(clock, 0.020, max_frames=4) for _ in range(2)]
    srv = serving.Server(slots, clock=clock)
    for i in range(16):
        clock.t = i * 0.002
        srv.submit(serving.Request(i, 0, _frame(1), clock.t))
        srv.poll()
    srv_launches = [n for s in slots for n in s.launches]
    assert max(srv_launches) > 1          # later arrivals were batched together
    assert srv.max_in_flight == 2         # both slots were on the "device" at once
    while not srv.idle():
        clock.t += 0.001
        srv.poll()
    assert len(srv.completed) == 16


def test_slot_budget_limits_a_batch():
    clock = FakeClock()
    slot = FakeExecutor(clock, 0.005, max_frames=8, max_pixels=200)
    srv = serving.Server([slot], clock=clock)
    for i in range(6):
        srv.submit(serving.Request(i, 0, _frame(1), 0.0))   # 64 px each: 3 fit in 200
    srv.poll()
    assert slot.launches == [3]


def test_admission_by_memory():
    assert serving.slots_for_memory(100 << 30, 10 << 30, fraction=0.5, max_slots=8) == 5
    assert serving.slots_for_memory(1 << 30, 10 << 30) == 1
    assert serving.slots_for_memory(1000 << 30, 1 << 30, max_slots=8) == 8


def test_poisson_arrivals_are_reproducible_and_at_the_right_rate():
    a = serving.poisson_arrivals([60, 30], 10.0, seed=1)
    b = serving.poisson_arrivals([60, 30], 10.0, seed=1)
    assert a == b
    n0 = sum(1 for _, c in a if c == 0)
    n1 = sum(1 for _, c in a if c == 1)
    assert 500 < n0 < 700 and 230 < n1 < 370
    assert all(a[i][0] <= a[i + 1][0] for i in range(len(a) - 1))


def test_camera_replay_in_real_time_with_idle_sleep():
    """run_cameras against the wall clock: with the loop sleeping while
    nothing is queued or in flight, every arrival is still served once, with
    its own result, and nothing waits on a sleeping loop for long."""
    import time
    clock = time.perf_counter
    slots = [FakeExecutor(clock, 0.0005) for _ in range(2)]
    srv = serving.Server(slots)
    cams = [[_frame(10 * c + k) for k in range(2)] for c in range(4)]
    before = serving.host_counters()
    res = serving.run_cameras(srv, cams, [200.0] * 4, duration_s=0.3, seed=5, idle_sleep=True)
    delta = serving.counter_delta(before, serving.host_counters())
    assert delta["involuntary_switches"] >= 0
    arrivals = serving.poisson_arrivals([200.0] * 4, 0.3, 5)
    assert [r.seq for r in res] == list(range(len(arrivals)))
    k = [0] * 4
    for r, (_, cam) in zip(res, arrivals):
        assert r.camera == cam
        assert int(r.quads[0]) == int(cams[cam][k[cam] % 2].sum())
        k[cam] += 1
    # a sleep ends 0.2 ms before the next arrival; allow for a slow host
    assert max(r.latency_ms for r in res) < 50.0

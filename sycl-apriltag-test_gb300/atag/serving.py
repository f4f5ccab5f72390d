"""Continuous-batching request loop for multi-camera quad detection.

Requests (one frame each, host memory) arrive at any time.  The server owns
a pool of *slots*; each slot is one in-flight micro-batch with its own CUDA
stream and a detector whose workspace (thresholded image, union-find forest,
labels, sizes, pair tables, cluster buffers) stays resident for the life of
the server.  The number of slots is chosen from the free device memory at
start-up (admission by memory), and each slot admits frames up to its pixel
budget.  Whenever a slot is free, every request that has arrived since is
admitted into it; slots run concurrently on the device, so requests that
arrive while others are on the GPU overlap with them.  Latency is measured
from arrival to the moment the slot's results are back on the host.

The scheduler is independent of CUDA: it drives objects with the Executor
interface (`launch`, `done`, `results`), so its logic is tested on the CPU
with a fake executor and run on the GPU with DetectorExecutor.
"""
import collections
import contextlib
import gc
import resource
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    seq: int
    camera: int
    frame: object              # H x W uint8, source resolution: a numpy array, or a
                               # pinned host tensor (a capture buffer) copied to the
                               # device without a host-side copy
    t_arrival: float           # seconds, on the server clock


def frame_pixels(frame) -> int:
    return int(frame.shape[0]) * int(frame.shape[1])


@dataclass
class Result:
    seq: int
    camera: int
    quads: np.ndarray          # QUAD_CORNERS records
    stats: np.void
    t_arrival: float
    t_done: float
    batch_size: int

    @property
    def latency_ms(self):
        return 1000.0 * (self.t_done - self.t_arrival)


class DetectorExecutor:
    """One slot on the GPU: resident detector + stream + pinned staging."""

    def __init__(self, max_width, max_height, max_frames, max_total_pixels, config=None, quad_capacity=256,
                 src_factor=1):
        import torch

        from .detector import Detector
        self.torch = torch
        self.det = Detector(max_width, max_height, max_frames=max_frames, max_total_pixels=max_total_pixels,
                            config=config, quad_capacity=quad_capacity)
        self.stream = torch.cuda.Stream()
        src_px = max_total_pixels * src_factor * src_factor
        self.h_in = torch.empty(src_px, dtype=torch.uint8).pin_memory()
        self.d_in = torch.empty(src_px, dtype=torch.uint8, device="cuda")
        self.h_stats = torch.empty(self.det.d_stats.numel(), dtype=torch.uint8).pin_memory()
        self.h_quads = torch.empty(self.det.d_quads.numel(), dtype=torch.uint8).pin_memory()
        self.event = torch.cuda.Event()
        self.max_frames = max_frames
        self.max_pixels = src_px
        self.n = 0
        self.max_enqueue_time = 0.0  # longest detector enqueue (host side of the launches)

    def capacity(self):
        return self.max_frames, self.max_pixels

    def launch(self, frames):
        torch = self.torch
        off = 0
        views = []
        with torch.cuda.stream(self.stream):
            for f in frames:
                n = frame_pixels(f)
                if isinstance(f, torch.Tensor) and f.is_pinned():
                    # a capture buffer in pinned memory: straight to the device
                    self.d_in[off:off + n].copy_(f.reshape(-1), non_blocking=True)
                else:
                    self.h_in[off:off + n].numpy()[:] = np.asarray(f).reshape(-1)
                    self.d_in[off:off + n].copy_(self.h_in[off:off + n], non_blocking=True)
                views.append((off, tuple(f.shape)))
                off += n
            dev = [self.d_in[o:o + s[0] * s[1]].view(s[0], s[1]) for o, s in views]
            t0 = time.perf_counter()
            self.det.enqueue(dev, stream=self.stream)
            self.max_enqueue_time = max(self.max_enqueue_time, time.perf_counter() - t0)
            self.h_stats.copy_(self.det.d_stats, non_blocking=True)
            self.h_quads.copy_(self.det.d_quads, non_blocking=True)
            self.event.record(self.stream)
        self.n = len(frames)

    def done(self):
        return self.event.query()

    def results(self):
        from .records import FRAME_STATS, QUAD_CORNERS
        self.event.synchronize()
        st = self.h_stats.numpy()[: self.n * FRAME_STATS.itemsize].view(FRAME_STATS)
        q = self.h_quads.numpy().view(QUAD_CORNERS).reshape(self.det.max_frames, self.det.quad_capacity)
        return [(q[i, : int(st[i]["n_quads"])].copy(), st[i].copy()) for i in range(self.n)]


def slots_for_memory(free_bytes, slot_bytes, fraction=0.5, max_slots=8):
    """Admission by device memory: how many resident slots fit in
    `fraction` of the free memory (at least one)."""
    return int(max(1, min(max_slots, (free_bytes * fraction) // max(slot_bytes, 1))))


def executor_bytes(max_width, max_height, max_frames, max_total_pixels, config=None, quad_capacity=256,
                   src_factor=1):
    """Device bytes one DetectorExecutor keeps resident: the detector's
    workspace (atag_workspace_size), its quad and stats buffers and the
    input staging buffer."""
    import ctypes

    from . import lib
    from .records import FRAME_STATS, QUAD_CORNERS
    L = lib.init()
    cfg = config or lib.default_config()
    size = ctypes.c_size_t()
    lib.check(L.atag_workspace_size(ctypes.byref(cfg), max_width, max_height, max_frames, max_total_pixels,
                                    ctypes.byref(size)), "atag_workspace_size")
    return (size.value + max_total_pixels * src_factor * src_factor +
            max_frames * (quad_capacity * QUAD_CORNERS.itemsize + FRAME_STATS.itemsize))


def executors_for_memory(max_width, max_height, max_frames, max_total_pixels, config=None, quad_capacity=256,
                         src_factor=1, fraction=0.5, max_slots=8):
    """As many DetectorExecutors as fit in `fraction` of the device's free
    memory (at most `max_slots`, at least one)."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    need = executor_bytes(max_width, max_height, max_frames, max_total_pixels, config, quad_capacity, src_factor)
    n = slots_for_memory(free, need, fraction, max_slots)
    return [DetectorExecutor(max_width, max_height, max_frames, max_total_pixels, config, quad_capacity, src_factor)
            for _ in range(n)]


class Server:
    """Continuous batching over a pool of executors (slots)."""

    def __init__(self, executors, clock=time.perf_counter):
        self.slots = list(executors)
        self.busy = [None] * len(self.slots)   # list of requests in flight per slot
        self.queue = collections.deque()
        self.clock = clock
        self.t0 = clock()
        self.completed = []
        self.max_in_flight = 0
        self.max_poll_gap = 0.0  # longest time between two polls (host stalls)
        self.max_poll_time = 0.0  # longest single poll (launches, result copies, stalls inside it)
        self.max_launch_time = 0.0  # longest launch of one slot (copies in, detector enqueue, copies out)
        self.max_results_time = 0.0  # longest read of one finished slot's results
        self._last_poll = None

    def now(self):
        return self.clock() - self.t0

    def submit(self, req: Request):
        self.queue.append(req)

    def _admit(self):
        for i, ex in enumerate(self.slots):
            if self.busy[i] is not None or not self.queue:
                continue
            max_frames, max_pixels = ex.capacity()
            take, px = [], 0
            while self.queue and len(take) < max_frames and px + frame_pixels(self.queue[0].frame) <= max_pixels:
                r = self.queue.popleft()
                take.append(r)
                px += frame_pixels(r.frame)
            if not take:  # a single frame larger than the slot's budget
                raise ValueError("frame exceeds the slot pixel budget")
            t0 = self.clock()
            ex.launch([r.frame for r in take])
            self.max_launch_time = max(self.max_launch_time, self.clock() - t0)
            self.busy[i] = take
        self.max_in_flight = max(self.max_in_flight, sum(b is not None for b in self.busy))

    def _reap(self):
        for i, ex in enumerate(self.slots):
            reqs = self.busy[i]
            if reqs is None or not ex.done():
                continue
            t0 = self.clock()
            out = ex.results()
            self.max_results_time = max(self.max_results_time, self.clock() - t0)
            t = self.now()
            for r, (quads, stats) in zip(reqs, out):
                self.completed.append(Result(r.seq, r.camera, quads, stats, r.t_arrival, t, len(reqs)))
            self.busy[i] = None

    def poll(self):
        t = self.clock()
        if self._last_poll is not None:
            self.max_poll_gap = max(self.max_poll_gap, t - self._last_poll)
        self._reap()
        self._admit()
        self._last_poll = self.clock()
        self.max_poll_time = max(self.max_poll_time, self._last_poll - t)

    def idle(self):
        return not self.queue and all(b is None for b in self.busy)

    def mark_resumed(self):
        """After a deliberate sleep: the gap since the last poll is not a stall."""
        self._last_poll = self.clock()

    def drain(self, timeout_s=60.0):
        end = self.now() + timeout_s
        while not self.idle():
            self.poll()
            if self.now() > end:
                raise TimeoutError("server did not drain")


@dataclass(order=True)
class _Arrival:
    t: float
    seq: int
    camera: int = field(compare=False)


def poisson_arrivals(rates_hz, duration_s, seed):
    """Merged Poisson arrival times of several cameras: [(t, camera)]."""
    rng = np.random.default_rng(seed)
    heap = []
    for cam, rate in enumerate(rates_hz):
        t = rng.exponential(1.0 / rate)
        while t < duration_s:
            heap.append((t, cam))
            t += rng.exponential(1.0 / rate)
    heap.sort()
    return heap


@contextlib.contextmanager
def latency_critical():
    """For the length of a serving run: one full garbage collection up front,
    then automatic collection off until the run ends.  The loop allocates a
    result record per request; with the collector on, its oldest generation
    is collected every so often over all the results kept so far, which in a
    minute-long run stalled a poll for up to ~60 ms (inside `poll`, so the
    gap between polls did not show it).  The objects that exist before the
    run are also frozen, so the collection after it skips them."""
    gc.collect()
    gc.freeze()
    gc.disable()
    try:
        yield
    finally:
        gc.enable()
        gc.unfreeze()


def host_counters():
    """Host-side counters that explain stalls of the request loop: this
    process's involuntary context switches (the scheduler took the CPU away)
    and, where the cgroup exposes them, the times the process's CPU quota
    was exhausted and its threads throttled."""
    out = {"involuntary_switches": resource.getrusage(resource.RUSAGE_SELF).ru_nivcsw}
    for path in ("/sys/fs/cgroup/cpu.stat", "/sys/fs/cgroup/cpu/cpu.stat", "/sys/fs/cgroup/cpu,cpuacct/cpu.stat"):
        try:
            with open(path) as f:
                for line in f:
                    k, _, v = line.partition(" ")
                    if k in ("nr_throttled", "throttled_usec", "throttled_time"):
                        out["cgroup_" + k] = int(v)
            break
        except (OSError, ValueError):
            continue
    return out


def counter_delta(before, after):
    return {k: after[k] - before[k] for k in after if k in before}


def warm(server: Server, frame):
    """Runs one frame through every slot before the clock starts (the first
    launch on a slot pays for lazy kernel loading and first-touch costs)."""
    for ex in server.slots:
        ex.launch([frame])
        ex.results()


def run_cameras(server: Server, camera_frames, rates_hz, duration_s, seed=0, on_result=None, idle_sleep=True):
    """Replays Poisson arrivals in real time: camera c submits
    camera_frames[c][k % len] at each of its arrival times.  Returns the
    completed results sorted by sequence number.  With idle_sleep, the loop
    sleeps while nothing is queued or in flight until shortly before the
    next arrival instead of spinning, so it holds a CPU only while it has
    work (a loop that spins all the time is the first thread a busy host
    preempts)."""
    arrivals = poisson_arrivals(rates_hz, duration_s, seed)
    counters = collections.Counter()
    seq = 0
    i = 0
    with latency_critical():
        server.t0 = server.clock()
        while i < len(arrivals):
            while True:
                wait = arrivals[i][0] - server.now()
                if wait <= 0:
                    break
                server.poll()
                if idle_sleep and wait > 3e-4 and server.idle():
                    time.sleep(wait - 2e-4)
                    server.mark_resumed()
            # every request whose arrival time has passed (several, when the
            # loop was busy launching) is queued with that arrival time, so
            # the time a request waits for the loop counts in its latency
            now = server.now()
            while i < len(arrivals) and arrivals[i][0] <= now:
                t, cam = arrivals[i]
                frames = camera_frames[cam]
                server.submit(Request(seq, cam, frames[counters[cam] % len(frames)], t))
                counters[cam] += 1
                seq += 1
                i += 1
            server.poll()
        server.drain()
    return sorted(server.completed, key=lambda r: r.seq)


def run_bursts(server: Server, camera_frames, n_bursts, burst_size, period_s, on_result=None):
    """Bursts of burst_size simultaneous requests (cameras taken in turn)
    every period_s seconds, e.g. a rig of cameras triggered together.
    Returns the completed results sorted by sequence number."""
    counters = collections.Counter()
    seq = 0
    with latency_critical():
        server.t0 = server.clock()
        for b in range(n_bursts):
            t = b * period_s
            while server.now() < t:
                server.poll()
            now = server.now()
            for k in range(burst_size):
                cam = seq % len(camera_frames)
                frames = camera_frames[cam]
                server.submit(Request(seq, cam, frames[counters[cam] % len(frames)], now))
                counters[cam] += 1
                seq += 1
            server.poll()
        server.drain()
    return sorted(server.completed, key=lambda r: r.seq)


def latency_summary(results, duration_s):
    lat = np.array([r.latency_ms for r in results]) if results else np.zeros(1)
    return {"requests": len(results), "frames_per_s": len(results) / duration_s,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "mean_batch": float(np.mean([r.batch_size for r in results]) if results else 0),
            "max_batch": int(max((r.batch_size for r in results), default=0)),
            "over_10ms": int((lat > 10.0).sum())}

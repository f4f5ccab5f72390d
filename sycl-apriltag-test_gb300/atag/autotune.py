"""Autotuner for the detector's launch shapes (atag_tuning).

Coordinate descent over a small space of tile and block shapes: starting
from the current shapes, each parameter in turn is set to every candidate
value with the others fixed, the detector is timed on the caller's frames
(one detect call captured as a CUDA graph, `reps` replays between CUDA
events after a warm-up) and the fastest value is kept; the sweep repeats
until nothing changes or `passes` run out.
Every shape gives bit-identical results, so tuning only changes speed.
Results are cached in a JSON file keyed by GPU, SM count, decimation and
the batch's frame sizes.
"""
import json
import os

SPACE = {
    "ccl_tile_rows": [8, 16, 32],
    "boundary_tile_rows": [8, 16],
    "small_cluster_max": [512, 1024, 2048],
    "small_ctas_per_sm": [4, 8, 12],
    "large_ctas_divisor": [1, 2, 4],
    "index_ctas_per_sm": [4, 8, 16],
    "batch_lanes": [1, 2, 3, 4],
}


def coordinate_descent(measure, start: dict, space=SPACE, passes=2):
    """Minimises measure(tuning) -> ms; returns (best tuning, best ms, log)."""
    best = dict(start)
    best_ms = measure(best)
    log = [(dict(best), best_ms)]
    for _ in range(passes):
        changed = False
        for name, values in space.items():
            for v in values:
                if v == best[name]:
                    continue
                cand = dict(best)
                cand[name] = v
                ms = measure(cand)
                log.append((cand, ms))
                if ms < best_ms:
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    return best, best_ms, log


def workload_key(det, frames):
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    shapes = sorted({tuple(f.shape) for f in frames})
    return f"{p.name}|{p.multi_processor_count}|d{det.cfg.decimate}|{len(frames)}x" + ",".join(
        f"{w}x{h}" for h, w in shapes)


def measure_fn(det, frames, reps=5):
    """Milliseconds per detect call of `det` on `frames` under a tuning: the
    call is captured as a CUDA graph and replayed `reps` times back to back,
    the way a batched caller runs it."""
    import torch
    stream = torch.cuda.Stream()

    def measure(tuning):
        det.set_tuning(**tuning)
        with torch.cuda.stream(stream):
            det.enqueue(frames, stream=stream)  # warm-up
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            det.enqueue(frames, stream=stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            graph.replay()
            a.record(stream)
            for _ in range(reps):
                graph.replay()
            b.record(stream)
        b.synchronize()
        del graph
        return a.elapsed_time(b) / reps
    return measure


def autotune(det, frames, reps=5, passes=2, cache_path=None):
    """Tunes `det` for `frames` (list of uint8 CUDA tensors), applies the best
    shapes, stores them in cache_path (if given) and returns
    {"tuning", "ms", "default_ms", "key", "tried"}."""
    start = det.get_tuning()
    measure = measure_fn(det, frames, reps)
    default_ms = measure(start)
    best, best_ms, log = coordinate_descent(measure, start, passes=passes)
    det.set_tuning(**best)
    key = workload_key(det, frames)
    if cache_path:
        cache = {}
        if os.path.exists(cache_path):
            with open(cache_path) as f:
                cache = json.load(f)
        cache[key] = best
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return {"tuning": best, "ms": best_ms, "default_ms": default_ms, "key": key, "tried": len(log)}


def apply_cached(det, frames, cache_path) -> bool:
    """Applies cached shapes for this GPU and workload if present."""
    if not cache_path or not os.path.exists(cache_path):
        return False
    with open(cache_path) as f:
        cache = json.load(f)
    t = cache.get(workload_key(det, frames))
    if t is None:
        return False
    det.set_tuning(**t)
    return True

"""Replicas across GPUs: one process per GPU, frames sharded by index, no
collective on the data path.

Frames are the independent units of quad detection (the reference's
`main()` handles one frame at a time, src/main.cpp:239-1030, and nothing
crosses frames), so a job of `world` ranks gives rank r the frames
r, r + world, r + 2·world, ...  Each rank runs its own detector on its own
device.  The only collectives are host-side bookkeeping: the max of the
ranks' timings (so a job's throughput is whole-job frames over the slowest
rank's time) and, for checking, the gather of per-frame results by global
frame index.  They run on whichever process group the job opened (NCCL on
GPUs, gloo on CPUs).
"""


def shard(n_frames, world, rank):
    """Global frame indices that `rank` processes (round-robin)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a job of {world}")
    return list(range(rank, n_frames, world))


def job_frames(frames_per_rank, world, rank):
    """Indices of a job in which every rank holds `frames_per_rank` frames."""
    return shard(frames_per_rank * world, world, rank)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value, device="cpu"):
    """Largest `value` over all ranks (the value itself without a job)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device="cpu"):
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.item()


def gather_by_index(indices, results):
    """All ranks' (global index, result) pairs merged into one list ordered
    by global frame index; every rank receives the whole list.  Raises if
    an index is missing or was processed twice."""
    local = list(zip(indices, results))
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        parts = [local]
    else:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
    merged = {}
    for part in parts:
        for i, r in part:
            if i in merged:
                raise ValueError(f"frame {i} processed by two ranks")
            merged[i] = r
    n = len(merged)
    if sorted(merged) != list(range(n)):
        raise ValueError("frames missing from the job")
    return [merged[i] for i in range(n)]

"""Rank body of the two-process replica test (gloo on CPU).  Each rank
detects its shard of the frames with the oracle (standing in for its GPU's
detector: the CUDA path needs a GPU), then the host logic gathers the
per-frame results by global index and reduces timings over ranks."""
import os
import sys


def run(rank, world, port, frames, out_dir):
    import numpy as np
    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "sycl-apriltag-test_gb300"))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import oracle
    from atag import replicas

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        cfg = oracle.default_config(decimate=2)
        idx = replicas.shard(len(frames), world, rank)
        mine = [oracle.detect(frames[i], cfg)["quads"] for i in idx]
        merged = replicas.gather_by_index(idx, mine)
        t_max = replicas.max_over_ranks(1.5 + rank)
        n_sum = replicas.sum_over_ranks(len(idx))
        # a shard that drops a frame is caught on every rank
        try:
            replicas.gather_by_index(idx[1:] if rank == 0 else idx, mine[1:] if rank == 0 else mine)
            missing = "not detected"
        except ValueError as e:
            missing = str(e)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), t_max=t_max, n_sum=n_sum, missing=missing,
                 **{f"q{i}": q for i, q in enumerate(merged)})
    finally:
        dist.destroy_process_group()

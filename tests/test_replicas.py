"""Replicas across GPUs, host side: frame sharding, gather by global frame
index and max-over-ranks timing, run as two gloo ranks on the CPU."""
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

import oracle
from atag import replicas
from conftest import synth_frame

import replicas_worker


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_partitions_frames():
    for n in (0, 1, 7, 64):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, world, r) for r in range(world)]
            flat = sorted(i for p in parts for i in p)
            assert flat == list(range(n))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    assert replicas.job_frames(4, 2, 1) == [1, 3, 5, 7]
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_single_process_needs_no_job():
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.gather_by_index([0, 1], ["a", "b"]) == ["a", "b"]
    with pytest.raises(ValueError):
        replicas.gather_by_index([1], ["a"])


def test_two_ranks_match_one_process(tmp_path):
    frames = [synth_frame("vga", s) for s in range(5)]
    world = 2
    tmp.start_processes(replicas_worker.run, args=(world, _free_port(), frames, str(tmp_path)),
                        nprocs=world, join=True, start_method="spawn")
    cfg = oracle.default_config(decimate=2)
    alone = [oracle.detect(f, cfg)["quads"] for f in frames]
    assert sum(len(q) for q in alone) > 0
    for rank in range(world):
        with np.load(tmp_path / f"rank{rank}.npz") as z:
            assert float(z["t_max"]) == 2.5
            assert int(z["n_sum"]) == len(frames)
            assert "missing" in str(z["missing"])
            for i, q in enumerate(alone):
                assert z[f"q{i}"].tobytes() == q.tobytes()

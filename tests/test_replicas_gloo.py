"""Multi-rank aggregation of bench.py, run as two gloo ranks on the CPU.

The hot path does not shard: N GPUs run N independent replicas, so the only
cross-rank step is the max-over-ranks time and the whole-job throughput
world * units / max_time.  These tests run that step with world_size 2.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, times, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], world)
        v = bench.replica_throughput(1000, t, world)
        with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
            f.write(f"{t!r} {v!r}\n")
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_world2(tmp_path):
    import torch.multiprocessing as mp
    times = [0.25, 0.5]
    mp.start_processes(_rank_main, args=(2, _free_port(), times, str(tmp_path)), nprocs=2,
                       join=True, start_method="spawn")
    for r in range(2):
        t, v = map(float, open(tmp_path / f"r{r}.txt").read().split())
        assert t == 0.5  # every rank sees the slowest replica
        assert v == pytest.approx(2 * 1000 / 0.5)


def test_single_rank_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.125, 1) == 0.125
    assert bench.replica_throughput(839619, 1e-4, 1) == pytest.approx(8.39619e9)

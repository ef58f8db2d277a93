"""The bench's multi-process path on the CPU: two gloo ranks reduce their
step times (max) and node counts (sum) the way the GPU ranks do over NCCL,
and each rank solves its own seeded batch (weak scaling, no data
collective)."""
import json
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    times = [10.0 + 5 * rank, 3.0 - rank]       # ms per rank
    work = [1000 * (rank + 1), 7]
    mx, sm = bench.job_max_sum(times, work, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "r%d.json" % rank), "w") as f:
        json.dump({"max": mx, "sum": sm}, f)


def test_two_gloo_ranks_reduce_like_the_bench(tmp_path):
    world, port = 2, _free_port()
    mp.start_processes(_rank, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn")
    for r in range(world):
        d = json.load(open(tmp_path / ("r%d.json" % r)))
        assert d["max"] == [15.0, 3.0]
        assert d["sum"] == [3000.0, 14.0]


def test_single_rank_passes_values_through():
    assert bench.job_max_sum([4.0], [9], 1, "cpu") == ([4.0], [9.0])


def test_each_rank_gets_its_own_batch():
    w0, a = bench.workload(0, 8)
    w1, b = bench.workload(1, 8)
    assert w0 == w1 == 4 and a.shape == b.shape == (8, 16)
    assert not np.array_equal(a, b)

"""Multi-GPU bench path (replicas: one independent patch per rank, no collective on the data
path) on the CPU with two gloo ranks: the whole-job time is the slowest rank's, and the
throughput counts every rank's work."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    ms = bench.max_over_ranks(10.0 * (rank + 1), ws)
    val = bench.replica_value(1000, ws, ms)
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write(f"{ms} {val}")
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        ms, val = map(float, open(tmp_path / f"r{r}").read().split())
        assert ms == pytest.approx(20.0)                   # the slowest rank
        assert val == pytest.approx(2 * 1000 / 20e-3)      # both ranks' work / that time

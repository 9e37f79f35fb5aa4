"""bench.py's N-GPU replica aggregation, run as two gloo ranks on the CPU: the job's
throughput is every rank's rows over the slowest rank's time (no data-path collective)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_s = [0.5, 2.0][rank]          # rank 1 is the slowest
    local_rows = [1_000_000, 3_000_000][rank]
    t, gbs = bench.replica_throughput(local_s, local_rows, dist, "cpu")
    out[rank] = (t, gbs)
    dist.destroy_process_group()


def test_two_rank_replicas():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    for r in range(world):
        t, gbs = res[r]
        assert t == 2.0
        assert gbs == pytest.approx(8.0 * 4_000_000 / 2.0 / 1e9)


def test_single_replica():
    import bench

    t, gbs = bench.replica_throughput(0.25, 1_000_000)
    assert t == 0.25 and gbs == pytest.approx(8.0 * 1_000_000 / 0.25 / 1e9)

"""`bench.py --gpus N` runs N independent replicas (one rank per GPU, no
collective on the data path). Its timing is the slowest rank's and its value
counts every rank's cell updates; two gloo ranks on the CPU check the host
side of that: rank discovery from the launcher's environment, the max over
ranks, and the whole-job rate."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_info()
    ms = [120.0, 180.0, 150.0][rank]
    slowest = bench.max_over_ranks(ms, device="cpu")
    q.put((rank, r, w, local, slowest, bench.job_rate(8e6 * 3, w, slowest * 1e-3)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_replica_timing_is_the_slowest_rank_and_value_counts_every_rank(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(k, world, port, q)) for k in range(world)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=180) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (k, r, w, local, slowest, rate) in enumerate(out):
        assert (k, r, w, local) == (rank, rank, world, rank)
        assert slowest == 180.0
        assert rate == pytest.approx(8e6 * 3 * world / 0.180)


def test_one_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(42.0, device="cpu") == 42.0
    assert bench.job_rate(10.0, 1, 2.0) == 5.0

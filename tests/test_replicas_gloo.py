"""The multi-GPU path of bench.py runs one replica per rank over its own batch shard; only the
timings cross ranks.  This checks that host logic with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
        ms = bench.max_over_ranks(local_ms, dist, "cpu")
        w, x = bench.make_inputs(dict(bench.CFG, nbatch=2), seed_offset=bench.shard_seed_offset(rank))
        gathered = [torch.zeros(2) for _ in range(world)]
        dist.all_gather(gathered, torch.tensor([float(x.sum()), float(w.sum())]))
        out[rank] = (ms, bench.job_value(world, 256, 400, ms), [g.tolist() for g in gathered])
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_own_shards():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    ms0, v0, g0 = res[0]
    ms1, v1, _ = res[1]
    assert ms0 == ms1 == 15.0                      # max over ranks
    assert v0 == v1 == 2 * 256 * 400 / 0.015       # all ranks' images over the slowest time
    assert g0[0][0] != g0[1][0]                    # each rank generated a different input shard
    assert g0[0][1] == g0[1][1]                    # ... of the same dictionary (one model)

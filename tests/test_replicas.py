"""The multi-GPU path of bench.py is replicas only (independent wavefunctions, no exchange):
its aggregation over ranks, run as two gloo processes on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    line = {"metric": "m", "value": 0.0, "ms_per_step": 10.0 + 5.0 * rank,
            "e2e": {"value": 1000.0 - 100.0 * rank, "unit": "wf-steps/s"}}
    agg = bench.aggregate_over_ranks(line, batch=256)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, agg))


def test_replica_aggregation_two_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    for r in (0, 1):
        agg = got[r]
        assert agg["n_gpus"] == 2
        assert agg["ms_per_step"] == 15.0                      # the slowest rank
        assert abs(agg["value"] - 2 * 256 * 1e3 / 15.0) < 1e-9   # all ranks' work over that time
        assert abs(agg["e2e"]["value"] - 2 * 900.0) < 1e-9      # slowest rank's e2e, times the ranks

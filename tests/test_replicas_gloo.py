"""The multi-GPU path of bench.py is replicas only: each rank runs its own
plan and the only collective is the max of the per-rank step time.  Checked
here with two gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 10.0 + 5.0 * rank                       # rank 1 is the slow replica
    m = bench.max_over_ranks(ms, dist)
    out[rank] = (m, bench.replica_value(m, ws))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1] == (15.0, 2 * 1000.0 / 15.0)


def test_single_rank_needs_no_collective():
    import bench
    assert bench.max_over_ranks(7.5, None) == 7.5
    assert bench.replica_value(7.5, 1) == pytest.approx(1000.0 / 7.5)

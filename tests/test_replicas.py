"""The multi-GPU form is replicas (one process per GPU, independent pairs,
no collective on the data path); only the timing crosses ranks.  Two gloo
ranks on the CPU check the barrier, the maximum over ranks and the
whole-job rate that bench.py reports."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from mia_gb300 import replicas
    assert replicas.env() == (world, rank, rank)
    assert replicas.init("gloo") == world
    replicas.barrier()
    # rank r took 0.1 * (r + 1) s for 10 units
    rate, t = replicas.whole_job_rate(10.0, 0.1 * (rank + 1), world)
    m = replicas.max_over_ranks(float(rank))
    replicas.barrier()
    dist.destroy_process_group()
    out.put((rank, rate, t, m))


@pytest.mark.parametrize("world", [2])
def test_whole_job_rate_is_all_units_over_the_slowest_rank(world):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(world))
    slowest = 0.1 * world
    for rank, rate, t, m in res:
        assert t == pytest.approx(slowest)
        assert rate == pytest.approx(world * 10.0 / slowest)
        assert m == world - 1


def test_one_rank_needs_no_process_group(monkeypatch):
    from mia_gb300 import replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.env() == (1, 0, 0)
    assert replicas.init() == 1
    replicas.barrier()
    assert replicas.whole_job_rate(10.0, 0.5, 1) == (20.0, 0.5)

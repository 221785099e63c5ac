"""The multi-GPU path's host logic on CPU: two gloo ranks (world size 2) agree on the slowest rank's
step time and on the job's total units, as the benchmark reports them under torchrun; environment
shares cover every environment exactly once."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from difftactile_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world_size, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world_size),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        r, ws, lr = replicas.rank_info()
        ms = 10.0 + 5.0 * rank              # rank 1 is the slower one
        units = 1000 * (rank + 1)
        replicas.barrier()
        q.put((r, ws, lr, replicas.slowest(ms), replicas.total(units), list(replicas.shard(7, r, ws))))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time_and_the_total_units():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:3] for o in out] == [(0, 2, 0), (1, 2, 1)]
    assert all(o[3] == 15.0 for o in out)          # max over ranks
    assert all(o[4] == 3000.0 for o in out)        # sum over ranks
    assert out[0][5] + out[1][5] == list(range(7))  # disjoint, complete, contiguous shares


@pytest.mark.parametrize("n,ws", [(64, 8), (7, 2), (3, 4), (0, 2)])
def test_shards_partition_the_environments(n, ws):
    got = [list(replicas.shard(n, r, ws)) for r in range(ws)]
    assert sum(got, []) == list(range(n))
    sizes = [len(g) for g in got]
    assert max(sizes) - min(sizes) <= 1


def test_single_process_needs_no_group():
    assert replicas.slowest(3.5) == 3.5 and replicas.total(2) == 2.0

"""The multi-replica path of bench.py on the CPU: two ranks over gloo (the solve
does not shard; every rank runs its own replica and only the timing barrier and
the max-over-ranks reduction cross ranks).  Checks the rank / world reading,
the barrier and that every rank sees the largest per-rank time, so that
`value` = total solves / the slowest rank's time."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    r, w, loc = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    bench.barrier(w)
    t_max = bench.max_over_ranks(1.0 + rank, w)  # rank 1 is the slower one
    steps = 5
    value = steps * w / t_max
    bench.barrier(w)
    dist.destroy_process_group()
    out.put((r, w, loc, t_max, value))


def test_two_replicas_share_the_slowest_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[3] == pytest.approx(2.0) for r in res)
    assert all(r[4] == pytest.approx(5 * 2 / 2.0) for r in res)


def test_single_rank_defaults():
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_env() == (0, 1, 0)
    assert bench.max_over_ranks(3.5, 1) == 3.5

"""Replica logic across two processes with the gloo backend (CPU, no GPU)."""
import os
import socket

import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    from autopdex_gb300 import replicas
    seeds = list(range(11))
    mine = replicas.shard(seeds)
    t = replicas.max_over_ranks(1.5 + rank)
    total = replicas.sum_over_ranks(len(mine))
    out.put((rank, mine, t, total))
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()


def test_two_rank_shards_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, t0, n0), (r1, s1, t1, n1) = res
    assert s0 + s1 == list(range(11)) and not set(s0) & set(s1)
    assert abs(len(s0) - len(s1)) <= 1
    assert t0 == t1 == 2.5 and n0 == n1 == 11


def test_shard_without_process_group():
    from autopdex_gb300 import replicas
    assert replicas.shard(list(range(5)), 0, 1) == list(range(5))
    assert replicas.shard(list(range(5)), 1, 2) == [2, 3, 4]

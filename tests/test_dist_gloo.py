"""The replica host logic with two gloo ranks on CPU: distinct seeds per rank,
max-over-ranks timing, gathered energies."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from fricc_gb300 import dist as D
    from fricc_gb300.rng import GlibcRand
    w, r, lr = D.world()
    seed = D.replica_seed(1000, r)
    first = GlibcRand(seed).uniform()
    t = D.max_over_ranks(1.0 + r)
    vals = D.gather_values(first)
    q.put((r, w, seed, t, vals))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, s0, t0, v0), (r1, w1, s1, t1, v1) = res
    assert w0 == w1 == 2 and s0 != s1
    assert t0 == t1 == 2.0          # the slowest rank's interval
    assert v0 == v1 and v0[0] != v0[1]

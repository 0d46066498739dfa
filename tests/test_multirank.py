"""The multi-rank path on CPU: two gloo ranks, as bench.py runs N replicas
(one process per GPU, no data-path collective).  Checks the scene shares of
a batch and the whole-job rate (units of all ranks over the slowest rank)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from stardust_gb300 import replicas
        mine = replicas.shard(11, rank, world)
        # rank r processed 1000 * (r + 1) units in (r + 1) * 0.5 s
        rate = replicas.job_rate(1000.0 * (rank + 1), 0.5 * (rank + 1))
        tmax = replicas.max_over_ranks(0.5 * (rank + 1))
        q.put((rank, mine, rate, tmax))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    shares = [o[1] for o in out]
    assert sorted(shares[0] + shares[1]) == list(range(11)) and not set(shares[0]) & set(shares[1])
    assert abs(len(shares[0]) - len(shares[1])) <= 1
    for _, _, rate, tmax in out:
        assert tmax == pytest.approx(1.0)
        assert rate == pytest.approx(3000.0 / 1.0)


def test_shard_rejects_bad_rank():
    from stardust_gb300 import replicas
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)

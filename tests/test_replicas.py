"""N > 1 replica path on CPU: two gloo ranks agree on the slowest rank's time and split the
serving requests into disjoint shares that cover the mix."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from warpcfd_gb300.replicas import job_throughput, max_over_ranks, shard
        from warpcfd_gb300.serve import make_request_mix

        t = max_over_ranks(1.0 + rank)            # rank r took 1 + r seconds
        reqs = make_request_mix(11, seed=5, rate=100.0)
        mine = [r.rid for r in shard(reqs, rank, world)]
        q.put((rank, t, job_throughput(100.0, world, t), mine))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [2.0, 2.0]        # both see the slowest rank's time
    assert out[0][2] == pytest.approx(100.0)         # 2 ranks x 100 units / 2 s
    ids = out[0][3] + out[1][3]
    assert sorted(ids) == list(range(11)) and not set(out[0][3]) & set(out[1][3])
    assert abs(len(out[0][3]) - len(out[1][3])) <= 1


def test_single_process_defaults():
    from warpcfd_gb300.replicas import max_over_ranks, shard

    assert max_over_ranks(3.5) == 3.5
    assert shard(range(5), 0, 1) == [0, 1, 2, 3, 4]
    with pytest.raises(ValueError):
        shard(range(5), 2, 2)

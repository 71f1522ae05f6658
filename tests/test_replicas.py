"""Multi-rank (replica) logic on CPU: two gloo ranks over 127.0.0.1.

Each rank computes its shard of a matrix's source rows with the CPU oracle
(standing in for its GPU); rank 0 gathers the shards and checks them against
the full matrix, and the timing reduction takes the max over ranks. No
kernel runs here, and no rank waits on another except in the collectives."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, cch, src, tgt, want, q):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "butterfly-osm_gb300"), root):
        if p not in sys.path:
            sys.path.insert(0, p)
    import replicas
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b, e = replicas.shard(len(src), rank, world)
        rows, _ = orc.Cch.from_dict(cch).matrix(src[b:e], tgt)
        # the slowest rank sets the job time: rank r reports 10 + r
        t_max = replicas.max_over_ranks(10.0 + rank, dist)
        sizes = [None] * world
        dist.all_gather_object(sizes, (b, e, rows))
        ok = True
        if rank == 0:
            full = np.concatenate([r for _, _, r in sorted(sizes, key=lambda x: x[0])])
            ok = bool(np.array_equal(full, want)) and [x[:2] for x in sorted(sizes)] == [
                replicas.shard(len(src), r, world) for r in range(world)]
        q.put((rank, t_max, ok))
    finally:
        dist.destroy_process_group()


def test_shard_covers_units():
    import replicas
    for n in (0, 1, 7, 10, 10000):
        for world in (1, 2, 3, 8):
            spans = [replicas.shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            assert max(e - b for b, e in spans) - min(e - b for b, e in spans) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)
    assert replicas.whole_job_rate(100, 4, 2.0) == 200.0
    assert replicas.max_over_ranks(3.5) == 3.5


def test_two_gloo_ranks_shard_a_matrix(built, grid100):
    import workload
    from oracle import oracle as orc
    _, cch = grid100
    src, tgt = workload.sources_targets(cch["n"], 37, 50, seed=11)
    want, _ = orc.Cch.from_dict(cch).matrix(src, tgt)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, cch, src, tgt, want, q))
             for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in out) == [0, 1]
    assert all(t == 11.0 for _, t, _ in out)  # max over ranks of 10 + rank
    assert all(ok for _, _, ok in out)

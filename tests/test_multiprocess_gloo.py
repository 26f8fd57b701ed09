"""The multi-process host logic on CPU with the gloo backend (world size 2,
spawned processes, rendezvous on 127.0.0.1): the bench's reductions over
replicas (max of the times, sum of the work) and the deterministic
partition of independent chains over ranks (every rank computes the same
assignment; together the ranks cover every chain exactly once)."""
import os
import socket

import numpy as np
import pytest

WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, queue):
    try:
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        import torch.distributed as dist
        dist.init_process_group("gloo", rank=rank, world_size=WORLD)
        import bench
        from dmrgpy_gb300.batch import partition_chains
        t = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        w = bench.sum_over_ranks(10.0 * (rank + 1), dist, "cpu")
        rng = np.random.default_rng(7)
        chis = rng.choice([16, 32, 64, 128], 256)
        parts = partition_chains([c ** 3 for c in chis], WORLD)
        gathered = [None] * WORLD
        dist.all_gather_object(gathered, parts[rank])
        dist.barrier()
        dist.destroy_process_group()
        queue.put((rank, t, w, gathered, parts, [int(c) for c in chis]))
    except Exception as exc:  # pragma: no cover - reported to the parent
        queue.put((rank, "error", repr(exc)))


def test_gloo_replica_reductions_and_chain_partition():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, queue)) for r in range(WORLD)]
    for p in procs:
        p.start()
    results = []
    try:
        for _ in range(WORLD):
            results.append(queue.get(timeout=180))
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
    for r in results:
        assert r[1] != "error", r
    results.sort()
    for rank, t, w, gathered, parts, chis in results:
        assert t == 2.5                       # the slowest replica
        assert w == 30.0                      # all replicas' work
        assert gathered == parts              # every rank derived the same partition
    parts = results[0][4]
    chis = results[0][5]
    allidx = sorted(i for p in parts for i in p)
    assert allidx == list(range(len(chis)))   # each chain exactly once
    loads = [sum(chis[i] ** 3 for i in p) for p in parts]
    assert max(loads) - min(loads) <= 128 ** 3   # balanced to within one chain


def test_partition_chains_single_rank_and_ties():
    from dmrgpy_gb300.batch import partition_chains
    assert partition_chains([3, 1, 2], 1) == [[0, 1, 2]]
    assert partition_chains([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    assert partition_chains([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        partition_chains([1], 0)

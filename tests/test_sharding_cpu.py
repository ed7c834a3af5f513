"""Row-sharded LOF host logic on CPU ranks (gloo, world size 2 and 3): the
sharded plan with its two all-gathers reproduces the single-process scores
bit for bit. The per-rank compute is the CPU oracle (test infrastructure)."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from culof_gb300.sharding import shard_rows


def test_shard_rows_partition():
    for n in (2, 7, 100, 200_001):
        for world in (1, 2, 3, 8):
            blocks = [shard_rows(n, world, r) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            sizes = [e - b for b, e in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_rows(10, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, X, k, out):
    import torch.distributed as dist

    import oracle
    from culof_gb300.sharding import sharded_lof

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        Xc, _, _ = oracle.center(X)
        n = X.shape[0]

        def knn_rows(b, e):
            idx, d2, kd = oracle.knn(Xc, k, rows=(b, e), nthreads=1)
            return idx[:, b:e], d2[:, b:e], kd[b:e]

        def lrd_rows(idx, d2, kd_all):
            # LRD of local rows: reachability uses every neighbour's k-distance
            reach = np.maximum(kd_all[idx], d2).astype(np.float32)
            s = np.zeros(idx.shape[1], np.float64)
            for t in range(idx.shape[0]):
                s += np.sqrt(reach[t].astype(np.float64))
            return (1.0 / (s / k + 1e-10)).astype(np.float32)

        def score_rows(idx, lrd_local, lrd_all):
            s = np.zeros(idx.shape[1], np.float64)
            for t in range(idx.shape[0]):
                s += lrd_all[idx[t]].astype(np.float64) / lrd_local.astype(np.float64)
            return (s / k).astype(np.float32)

        scores = sharded_lof(n, knn_rows, lrd_rows, score_rows)
        if rank == 0:
            out.put(scores)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_plan_matches_single_process(world):
    import torch.multiprocessing as mp

    import oracle
    from culof_gb300 import synthetic

    X = synthetic.clusters_with_outliers(1500, 5, seed=31)
    k = 12
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, X, k, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    np.testing.assert_array_equal(got, oracle.lof(X, k))

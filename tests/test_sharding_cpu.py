"""Row-sharded LOF host logic on CPU ranks (gloo, world size 2 and 3): the
sharded plan with its all-reduce exchanges reproduces the single-process
scores bit for bit. The per-rank compute here is the CPU oracle (test
infrastructure) over blocks of original rows; the GPU tests drive the same
plan with the engine's shard entry points."""

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


def oracle_steps(X, k):
    """The plan's three per-rank steps on the CPU oracle (torch CPU tensors)."""
    import torch

    import oracle

    Xc, _, _ = oracle.center(X)
    n = X.shape[0]

    def knn_shard(shard, num_shards):
        b, e = shard_rows(n, num_shards, shard)
        rows = np.arange(b, e, dtype=np.int64)
        li, ld, lk = oracle.knn_list(Xc, k, rows, nthreads=1)
        idx = np.zeros((k, n), np.int32)
        d2 = np.zeros((k, n), np.float32)
        kd = np.zeros(n, np.float32)
        idx[:, rows], d2[:, rows], kd[rows] = li, ld, lk
        return idx, d2, torch.from_numpy(kd), rows

    def lrd_rows(idx, d2, kd_all, rows):
        sub_lrd = oracle.lrd(idx[:, rows], d2[:, rows], kd_all.numpy())
        out = np.zeros(n, np.float32)
        out[rows] = sub_lrd
        return torch.from_numpy(out)

    def score_rows(idx, lrd_all, rows):
        lrd = lrd_all.numpy()
        s = np.zeros(len(rows), np.float64)
        for t in range(k):
            s += lrd[idx[t, rows]].astype(np.float64) / lrd[rows].astype(np.float64)
        out = np.zeros(n, np.float32)
        out[rows] = (s / k).astype(np.float32)
        return torch.from_numpy(out)

    return knn_shard, lrd_rows, score_rows


def _worker(rank, world, port, X, k, out):
    import torch.distributed as dist

    from culof_gb300.sharding import dist_exchange, sharded_lof

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        scores = sharded_lof(rank, world, *oracle_steps(X, k), dist_exchange())
        out.put((rank, scores.numpy()))
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
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = oracle.lof(X, k)
    for r in range(world):  # every rank holds all n scores
        np.testing.assert_array_equal(got[r], want)


def test_thread_exchange_sums_in_rank_order():
    import threading

    import torch

    from culof_gb300.sharding import ThreadExchange

    ex = ThreadExchange(3)
    parts = [torch.tensor([1.0, 0.0, 0.0]), torch.tensor([0.0, 2.0, 0.0]), torch.tensor([0.0, 0.0, 3.0])]
    res = [None] * 3

    def run(r):
        res[r] = ex.for_rank(r)(parts[r])

    th = [threading.Thread(target=run, args=(r,)) for r in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=30)
    for r in range(3):
        assert res[r].tolist() == [1.0, 2.0, 3.0]

"""Row-sharded runs simulated on one GPU.

The shards of culof_context_knn_shard_device cover every row exactly once,
each row's neighbours equal the unsharded call's bit for bit, the LRD and
score row-block entry points complete the LOF, and the whole plan of
culof_gb300.sharding (two exchanges of n floats between the k-NN, the LRD
and the scores) run by 2 and 3 ranks as threads of one process gives the
single call's scores bit for bit at the plain exact-LOF workload's shape
(n = 200,000, d = 8, k = 20). Each rank's kernels run independently; only
the host-side exchange waits."""

from __future__ import annotations

import threading

import numpy as np
import pytest

from culof_gb300 import _culof, synthetic
from culof_gb300.sharding import EngineShard, ThreadExchange, sharded_lof

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    ("clusters_n200000_d8_k20", lambda: synthetic.clusters_with_outliers(200_000, 8, seed=1), 20, _culof.PATH_AUTO),
    ("factor_n20000_d32_tensor", lambda: synthetic.factor_model(20_000, 32, seed=7), 20, _culof.PATH_TENSOR),
    ("clusters_n9000_d16_wide", lambda: synthetic.clusters_with_outliers(9_000, 16, seed=8), 15, _culof.PATH_FAST),
    ("clusters_n3000_k70_general", lambda: synthetic.clusters_with_outliers(3_000, 8, seed=9), 70,
     _culof.PATH_GENERAL),
]


def _single(X, k, path):
    n, d = X.shape
    dx = torch.from_numpy(X).cuda()
    idx = torch.zeros((k, n), dtype=torch.int32, device="cuda")
    d2 = torch.zeros((k, n), device="cuda")
    kd = torch.zeros(n, device="cuda")
    with _culof.Context() as ctx:
        ctx.set_path(path)
        ctx.knn_device(dx.data_ptr(), n, d, k, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
        scores = ctx.lof(X, k)
        _, total = ctx.pair_stats()
    return idx.cpu().numpy(), d2.cpu().numpy(), kd.cpu().numpy(), scores, total


@pytest.mark.parametrize("shards", [2, 3])
@pytest.mark.parametrize("name,make,k,path", CASES, ids=[c[0] for c in CASES])
def test_shards_cover_rows_and_match_the_single_call(name, make, k, path, shards):
    X = make()
    n = X.shape[0]
    idx0, d20, kd0, scores0, total0 = _single(X, k, path)
    eng = EngineShard(torch.from_numpy(X).cuda(), k)
    eng.ctx.set_path(path)
    seen = np.zeros(n, np.int64)
    parts, kd_all, totals = [], torch.zeros(n, device="cuda"), 0.0
    for s in range(shards):
        idx, d2, kd, rows = eng.knn_shard(s, shards)
        totals += eng.ctx.pair_stats()[1]
        r = rows.cpu().numpy()
        seen[r] += 1
        np.testing.assert_array_equal(idx.cpu().numpy()[:, r], idx0[:, r])
        np.testing.assert_array_equal(d2.cpu().numpy()[:, r].view(np.uint32), d20[:, r].view(np.uint32))
        np.testing.assert_array_equal(kd.cpu().numpy()[r].view(np.uint32), kd0[r].view(np.uint32))
        kd_all += kd
        parts.append((idx, d2, rows))
    assert (seen == 1).all()
    # the small-d sweep's work splits with the rows (its unpruned pair count)
    assert totals == total0
    lrd_all = sum(eng.lrd_rows(i, d, kd_all, r) for i, d, r in parts)
    scores = sum(eng.score_rows(i, lrd_all, r) for i, _, r in parts)
    np.testing.assert_array_equal(scores.cpu().numpy().view(np.uint32), scores0.view(np.uint32))
    eng.close()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_plan_as_threads_matches_the_single_call(world):
    X = synthetic.clusters_with_outliers(200_000, 8, seed=1)
    with _culof.Context() as ctx:
        want = ctx.lof(X, 20)
    dX = torch.from_numpy(X).cuda()
    ex = ThreadExchange(world)
    out, errors = [None] * world, []

    def rank(r):
        try:
            eng = EngineShard(dX, 20)
            out[r] = sharded_lof(r, world, eng.knn_shard, eng.lrd_rows, eng.score_rows, ex.for_rank(r)).cpu().numpy()
            eng.close()
        except Exception as e:  # noqa: BLE001  (reported below)
            errors.append(e)
            ex._barrier.abort()

    threads = [threading.Thread(target=rank, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for r in range(world):
        np.testing.assert_array_equal(out[r].view(np.uint32), want.view(np.uint32))


def test_row_block_entry_points_reject_bad_arguments():
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    f = torch.zeros(16, device="cuda")
    with pytest.raises(ValueError, match="num_rows"):
        _culof.compute_lrd_rows(0, buf.data_ptr(), f.data_ptr(), f.data_ptr(), 4, 1, buf.data_ptr(), 5, f.data_ptr())
    with _culof.Context() as ctx, pytest.raises(ValueError, match="shard"):
        X = torch.zeros((8, 2), device="cuda")
        ctx.knn_shard_device(X.data_ptr(), 8, 2, 2, False, 2, 2, buf.data_ptr(), f.data_ptr(), f.data_ptr(),
                             buf.data_ptr())

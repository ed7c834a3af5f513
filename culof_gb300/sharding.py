"""Row-sharded exact LOF across ranks: the host-side plan and exchange.

The k-NN stage shards by rows with no communication: every rank holds the
whole centred X (6.4 MB at n=200k, d=8) and selects the neighbours of its own
contiguous row block. LOF then needs two exchanges, each an all-gather of n
floats: the k-distances (for the reachability distances of the LRD) and the
LRDs (for the scores). The contamination offset is an order statistic of all
n scores (gathered here; a radix-histogram all-reduce is the alternative).

``shard_rows`` fixes the row blocks, and ``sharded_lof`` runs the plan over any
``torch.distributed`` process group with per-rank k-NN / LRD / score
callbacks, so the host logic is testable on CPU ranks (gloo) against the
single-process result.
"""

from __future__ import annotations

from typing import Callable

import numpy as np


def shard_rows(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous row block [begin, end) of `rank`; blocks differ by at most one row."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def _all_gather_rows(local: np.ndarray, n: int, world: int, group=None) -> np.ndarray:
    """Concatenate every rank's row block (row blocks from shard_rows)."""
    import torch
    import torch.distributed as dist

    counts = [shard_rows(n, world, r)[1] - shard_rows(n, world, r)[0] for r in range(world)]
    width = max(counts)
    pad = np.zeros((width,) + local.shape[1:], local.dtype)
    pad[: local.shape[0]] = local
    t = torch.from_numpy(pad)
    out = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(out, t, group=group)
    return np.concatenate([o.numpy()[:c] for o, c in zip(out, counts)], axis=0)


def sharded_lof(
    n: int,
    knn_rows: Callable[[int, int], tuple[np.ndarray, np.ndarray, np.ndarray]],
    lrd_rows: Callable[[np.ndarray, np.ndarray, np.ndarray], np.ndarray],
    score_rows: Callable[[np.ndarray, np.ndarray, np.ndarray], np.ndarray],
    group=None,
) -> np.ndarray:
    """LOF scores of all n points, computed row-sharded over the process group.

    knn_rows(begin, end) -> (nbr_idx (k, m), nbr_d2 (k, m), kdist2 (m,)) for rows
    [begin, end); lrd_rows(nbr_idx, nbr_d2, kdist2_all) -> lrd (m,);
    score_rows(nbr_idx, lrd_local, lrd_all) -> scores (m,). Returns the gathered
    scores (every rank gets all n).
    """
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    b, e = shard_rows(n, world, rank)
    idx, d2, kd = knn_rows(b, e)
    kd_all = _all_gather_rows(np.ascontiguousarray(kd, np.float32), n, world, group)  # exchange 1
    lrd = lrd_rows(idx, d2, kd_all)
    lrd_all = _all_gather_rows(np.ascontiguousarray(lrd, np.float32), n, world, group)  # exchange 2
    scores = score_rows(idx, lrd, lrd_all)
    return _all_gather_rows(np.ascontiguousarray(scores, np.float32), n, world, group)

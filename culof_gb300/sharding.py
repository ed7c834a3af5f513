"""Row-sharded exact LOF across ranks (one process per GPU).

The plan (the reference splits the same stage into row tiles on one GPU,
src/cuda/pipeline.cu:175-195):

1. Every rank holds all n points and computes the k-NN of its shard of the
   rows against all n points, with no communication
   (``culof_context_knn_shard_device``: on the fused paths a shard is a block
   of the engine's spatial order, which every rank derives identically from
   the same points; on the general path a block of original rows).
2. Exchange 1: the k-distances (n floats), for the reachability distances of
   the LRD.
3. Each rank computes the LRD of its rows (``culof_compute_lrd_rows``).
4. Exchange 2: the LRDs (n floats), for the scores.
5. Each rank computes the scores of its rows (``culof_compute_scores_rows``);
   a third exchange gives every rank all n scores (the contamination offset
   is an order statistic of all of them).

Every entry of an exchanged array is written by exactly one shard and is
zero elsewhere, so each exchange is an all-reduce (sum) of n floats and is
exact (x + 0 = x), whatever order the reduction adds in.

``sharded_lof`` runs the plan with three per-rank steps and an exchange
function. ``EngineShard`` supplies the steps from the engine (CUDA tensors);
``dist_exchange`` is the all-reduce of a ``torch.distributed`` group (NCCL
for CUDA tensors, gloo for CPU tensors); ``ThreadExchange`` simulates ranks as
threads of one process (every rank's kernels run independently on one GPU;
only the host-side exchange waits).
"""

from __future__ import annotations

import threading
from typing import Callable

import numpy as np


def shard_rows(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous block [begin, end) of `rank` among n items; blocks differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    return n * rank // world, n * (rank + 1) // world


def sharded_lof(shard: int, num_shards: int, knn_shard: Callable, lrd_rows: Callable, score_rows: Callable,
                exchange: Callable):
    """LOF scores of all n points, computed row-sharded; this is rank `shard`.

    knn_shard(shard, num_shards) -> (nbr_idx, nbr_d2, kdist2, rows): the
    shard's neighbour slots (k x n, its columns written), kdist2 (n, zero
    outside its rows) and the list of its rows;
    lrd_rows(nbr_idx, nbr_d2, kdist2_all, rows) -> lrd (n, zero outside rows);
    score_rows(nbr_idx, lrd_all, rows) -> scores (n, zero outside rows);
    exchange(a) -> the element-wise sum of every rank's `a`.
    Returns all n scores (on every rank).
    """
    idx, d2, kd, rows = knn_shard(shard, num_shards)
    kd_all = exchange(kd)  # exchange 1
    lrd = lrd_rows(idx, d2, kd_all, rows)
    lrd_all = exchange(lrd)  # exchange 2
    return exchange(score_rows(idx, lrd_all, rows))


class EngineShard:
    """The three per-rank steps on the engine, for points X (a CUDA float32
    tensor n x d) on the current device, on the current CUDA stream."""

    def __init__(self, X, k: int, normalize: bool = False):
        import torch

        from . import _culof

        if not X.is_cuda or X.dtype != torch.float32 or X.dim() != 2:
            raise ValueError("EngineShard expects a 2-D float32 CUDA tensor")
        self._culof = _culof
        self.X = X.contiguous()
        self.n, self.d = self.X.shape
        self.k, self.normalize = int(k), bool(normalize)
        self.ctx = _culof.Context()
        self.stream = torch.cuda.current_stream(self.X.device).cuda_stream
        self.ctx.set_stream(self.stream)

    def close(self) -> None:
        self.ctx.close()

    def _zeros(self, shape, dtype):
        import torch

        return torch.zeros(shape, dtype=dtype, device=self.X.device)

    def knn_shard(self, shard: int, num_shards: int):
        import torch

        idx = self._zeros((self.k, self.n), torch.int32)
        d2 = self._zeros((self.k, self.n), torch.float32)
        kd = self._zeros(self.n, torch.float32)
        rows = torch.empty(self.n, dtype=torch.int32, device=self.X.device)
        m = self.ctx.knn_shard_device(self.X.data_ptr(), self.n, self.d, self.k, self.normalize, shard, num_shards,
                                      idx.data_ptr(), d2.data_ptr(), kd.data_ptr(), rows.data_ptr())
        return idx, d2, kd, rows[:m]

    def lrd_rows(self, idx, d2, kd_all, rows):
        import torch

        lrd = self._zeros(self.n, torch.float32)
        self._culof.compute_lrd_rows(self.stream, idx.data_ptr(), d2.data_ptr(), kd_all.data_ptr(), self.n, self.k,
                                     rows.data_ptr(), rows.numel(), lrd.data_ptr())
        return lrd

    def score_rows(self, idx, lrd_all, rows):
        import torch

        scores = self._zeros(self.n, torch.float32)
        self._culof.compute_scores_rows(self.stream, idx.data_ptr(), lrd_all.data_ptr(), self.n, self.k,
                                        rows.data_ptr(), rows.numel(), scores.data_ptr())
        return scores


def dist_exchange(group=None) -> Callable:
    """All-reduce (sum) over a torch.distributed group."""
    import torch.distributed as dist

    def exchange(t):
        out = t.clone()
        dist.all_reduce(out, op=dist.ReduceOp.SUM, group=group)
        return out

    return exchange


class ThreadExchange:
    """All-reduce (sum) among `world` threads of one process: each rank of a
    simulated run calls ``for_rank(r)``'s function with its array; the sum is
    taken on the host in rank order and returned on the caller's device."""

    def __init__(self, world: int):
        self.world = world
        self._barrier = threading.Barrier(world)
        self._slots: list = [None] * world

    def for_rank(self, rank: int) -> Callable:
        def exchange(t):
            import torch

            self._slots[rank] = t.cpu().numpy()  # synchronises the rank's stream
            self._barrier.wait()
            total = np.zeros_like(self._slots[0])
            for part in self._slots:
                total += part
            self._barrier.wait()  # every rank has read the slots
            return torch.from_numpy(total).to(t.device)

        return exchange

"""Batched LOF (culof_context_lof_batched_device): many independent problems
in one persistent launch, replayed from a CUDA graph. Every problem's scores
must be bit-identical to a single-problem call and to the CPU oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from culof_gb300 import _culof, synthetic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _batch(problems, ks, normalize, ctx, graphs=True):
    d = problems[0].shape[1]
    X = np.concatenate(problems).astype(np.float32)
    off = np.zeros(len(problems) + 1, np.int64)
    off[1:] = np.cumsum([len(p) for p in problems])
    dx = torch.from_numpy(X).cuda()
    ds = torch.full((len(X),), float("nan"), dtype=torch.float32, device="cuda")
    ctx.set_graphs(graphs)
    ctx.lof_batched_device(off, ks, dx.data_ptr(), d, normalize, ds.data_ptr())
    ctx.synchronize()
    return off, dx, ds


def _split(scores, off):
    return [scores[off[i]:off[i + 1]] for i in range(len(off) - 1)]


@pytest.mark.parametrize("normalize", [False, True])
def test_batched_matches_single_problem_and_oracle(normalize):
    probs, ks = synthetic.batched_problems(48, 16, seed=3, n_range=(128, 4000), k_range=(10, 40))
    if normalize:
        for i, p in enumerate(probs):
            p[:, i % 16] *= 25.0
    with _culof.Context() as ctx:
        off, _, ds = _batch(probs, ks, normalize, ctx)
        got = _split(ds.cpu().numpy(), off)
        for i, (p, k) in enumerate(zip(probs, ks)):
            one = ctx.lof(p, k, normalize)
            np.testing.assert_array_equal(got[i].view(np.uint32), one.view(np.uint32))
            if i % 8 == 0:
                np.testing.assert_array_equal(got[i].view(np.uint32), oracle.lof(p, k, normalize).view(np.uint32))


def test_batched_edge_shapes():
    # n = 2 (k = 1), a one-row last tile, n = k + 1, d = 1 and d = 64 batches
    rng = np.random.default_rng(5)
    for d in (1, 3, 64):
        probs = [rng.standard_normal((n, d)).astype(np.float32) for n in (2, 129, 49, 300, 1000)]
        ks = [1, 20, 48, 7, 33]
        with _culof.Context() as ctx:
            off, _, ds = _batch(probs, ks, False, ctx)
            got = _split(ds.cpu().numpy(), off)
            for i, (p, k) in enumerate(zip(probs, ks)):
                np.testing.assert_array_equal(got[i].view(np.uint32), oracle.lof(p, k).view(np.uint32))


def test_graph_replay_reads_current_data_and_replans():
    probs, ks = synthetic.batched_problems(20, 16, seed=4, n_range=(200, 2000))
    with _culof.Context() as ctx:
        off, dx, ds = _batch(probs, ks, False, ctx)
        first = ds.cpu().numpy().copy()
        # same layout and pointers: replay
        ctx.lof_batched_device(off, ks, dx.data_ptr(), 16, False, ds.data_ptr())
        ctx.synchronize()
        np.testing.assert_array_equal(ds.cpu().numpy(), first)
        # new values in the same buffer: the replay must see them
        probs2 = [p * 0.5 + 1.0 for p in synthetic.batched_problems(20, 16, seed=9, n_range=(200, 2000))[0]]
        probs2 = [np.resize(q, p.shape).astype(np.float32) for p, q in zip(probs, probs2)]
        dx.copy_(torch.from_numpy(np.concatenate(probs2)).cuda())
        ctx.lof_batched_device(off, ks, dx.data_ptr(), 16, False, ds.data_ptr())
        ctx.synchronize()
        got = _split(ds.cpu().numpy(), off)
        for i in (0, 7, 19):
            np.testing.assert_array_equal(got[i], ctx.lof(probs2[i], ks[i]))
        # a different layout: re-plan
        ks3 = [min(k + 1, 48) for k in ks]
        ctx.lof_batched_device(off, ks3, dx.data_ptr(), 16, False, ds.data_ptr())
        ctx.synchronize()
        got = _split(ds.cpu().numpy(), off)
        for i in (3, 11):
            np.testing.assert_array_equal(got[i], ctx.lof(probs2[i], ks3[i]))


def test_batched_without_graphs_matches():
    probs, ks = synthetic.batched_problems(16, 16, seed=6, n_range=(128, 1500))
    with _culof.Context() as ctx:
        off, _, a = _batch(probs, ks, False, ctx, graphs=True)
        a = a.cpu().numpy()
    with _culof.Context() as ctx:
        _, _, b = _batch(probs, ks, False, ctx, graphs=False)
    np.testing.assert_array_equal(a, b.cpu().numpy())


def test_batched_validation():
    p = np.random.default_rng(1).standard_normal((50, 4)).astype(np.float32)
    dx = torch.from_numpy(np.concatenate([p, p])).cuda()
    ds = torch.empty(100, device="cuda")
    with _culof.Context() as ctx:
        with pytest.raises(ValueError, match="k must satisfy"):
            ctx.lof_batched_device([0, 50, 100], [50, 5], dx.data_ptr(), 4, False, ds.data_ptr())
        with pytest.raises(ValueError, match="k must satisfy"):
            ctx.lof_batched_device([0, 50, 100], [49, 5], dx.data_ptr(), 4, False, ds.data_ptr())
        with pytest.raises(ValueError, match="offsets"):
            ctx.lof_batched_device([1, 50, 100], [5, 5], dx.data_ptr(), 4, False, ds.data_ptr())
        with pytest.raises(ValueError, match="n_dims"):
            ctx.lof_batched_device([0, 50, 100], [5, 5], dx.data_ptr(), 65, False, ds.data_ptr())


def test_batched_problem_mix_subset_bit_exact():
    # 2,048 problems, n log-uniform in [128, 16384], d = 16, k in [10, 40]
    probs, ks = synthetic.batched_problems(2048, 16, seed=0)
    with _culof.Context() as ctx:
        off, _, ds = _batch(probs, ks, False, ctx)
        got = _split(ds.cpu().numpy(), off)
        rng = np.random.default_rng(2)
        for i in rng.choice(len(probs), 24, replace=False):
            np.testing.assert_array_equal(got[i].view(np.uint32), ctx.lof(probs[i], ks[i]).view(np.uint32))


def test_package_lof_batched_host_arrays():
    import culof_gb300

    probs, ks = synthetic.batched_problems(12, 16, seed=11, n_range=(128, 2000))
    got = culof_gb300.lof_batched(probs, ks)
    for p, k, g in zip(probs, ks, got):
        np.testing.assert_array_equal(g, culof_gb300.lof(p, k))
    same_k = culof_gb300.lof_batched(probs[:3], 15)
    for p, g in zip(probs[:3], same_k):
        np.testing.assert_array_equal(g, culof_gb300.lof(p, 15))
    with pytest.raises(ValueError):
        culof_gb300.lof_batched(probs[:2], [10])


def test_autotuner_record_names_the_fastest_variant():
    torch = pytest.importorskip("torch")
    probs, ks = synthetic.batched_problems(48, 16, seed=3)
    Xb = np.concatenate(probs).astype(np.float32)
    offs = np.zeros(len(probs) + 1, np.int64)
    offs[1:] = np.cumsum([len(p) for p in probs])
    with _culof.Context() as ctx:
        assert ctx.batched_tuning()["ctas_per_sm"] == 0  # nothing tuned yet
        dX = torch.from_numpy(Xb).cuda()
        ds = torch.empty(len(Xb), device="cuda")
        ctx.lof_batched_device(offs, ks, dX.data_ptr(), 16, False, ds.data_ptr())
        ctx.synchronize()
        tune = ctx.batched_tuning()
    assert tune["ctas_per_sm"] in (1, 2) and tune["pairs_per_lane"] in (1, 2)
    assert tune["ms"] and all(v > 0 for v in tune["ms"].values())
    chosen = f"{tune['ctas_per_sm']}cta_{tune['pairs_per_lane']}pair"
    assert tune["ms"][chosen] == min(tune["ms"].values())

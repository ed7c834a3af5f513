"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer/index outputs (neighbour indices, k-distance bits, labels) and every
float output are compared BIT FOR BIT: the engine and the oracle compute the
same float32 direct-difference distances, the same exact select and tie rule
(knn.cu:190-224), and the same FP64 LRD/score sums (lof.cu:32-62).
"""

from __future__ import annotations

import numpy as np
import pytest
from conftest import golden_case_arrays, rel_err

import oracle
from culof_gb300 import _culof, synthetic

pytestmark = pytest.mark.gpu

PATHS = [_culof.PATH_AUTO, _culof.PATH_GENERAL]
# every k-NN case also runs through each forced fused path that supports it
KNN_PATHS = [_culof.PATH_AUTO, _culof.PATH_GENERAL, _culof.PATH_FAST, _culof.PATH_TENSOR]


def torch_cuda():
    import torch

    return torch


def dev(a: np.ndarray):
    torch = torch_cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t) -> np.ndarray:
    return t.cpu().numpy()


@pytest.fixture
def ctx():
    c = _culof.Context()
    yield c
    c.close()


def run_knn(ctx, X, k, normalize=False):
    torch = torch_cuda()
    n, d = X.shape
    dx = dev(X)
    idx = torch.full((k, n), -1, dtype=torch.int32, device="cuda")
    d2 = torch.full((k, n), float("nan"), dtype=torch.float32, device="cuda")
    kd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    ctx.knn_device(dx.data_ptr(), n, d, k, normalize, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
    ctx.synchronize()
    return host(idx), host(d2), host(kd)


KNN_CASES = [
    ("clusters", lambda: synthetic.clusters_with_outliers(4000, 8, seed=1), 20),
    ("clusters_k1", lambda: synthetic.clusters_with_outliers(3000, 8, seed=2), 1),
    ("lowdim", lambda: synthetic.reference_test_data(400, 3, seed=11, n_outliers=8), 20),
    ("highdim", lambda: synthetic.reference_test_data(512, 32, seed=3, n_outliers=10), 15),
    ("d5_k25", lambda: synthetic.reference_test_data(700, 5, seed=13, n_outliers=9), 25),
    ("d16", lambda: synthetic.reference_test_data(3000, 16, seed=1, n_outliers=30), 10),
    ("d64", lambda: synthetic.reference_test_data(1500, 64, seed=2, n_outliers=15), 35),
    ("largek", lambda: synthetic.reference_test_data(600, 4, seed=5, n_outliers=12), 257),
    ("k_n_minus_1", lambda: synthetic.reference_test_data(128, 2, seed=7, n_outliers=4), 127),
    ("n2", lambda: np.array([[0.0, 1.0], [3.0, -1.0]], np.float32), 1),
    ("ragged", lambda: synthetic.clusters_with_outliers(1001, 7, seed=4), 33),
    ("dups", lambda: np.repeat(np.random.default_rng(4).standard_normal((50, 2)).astype(np.float32), 20, axis=0), 20),
    # fast-path shapes: one tile, a one-row last tile, lists of 128, d = 1
    ("n128", lambda: synthetic.clusters_with_outliers(128, 8, seed=21), 20),
    ("n129", lambda: synthetic.clusters_with_outliers(129, 8, seed=22), 20),
    ("k64", lambda: synthetic.clusters_with_outliers(5000, 8, seed=23), 64),
    ("k33_d3", lambda: synthetic.clusters_with_outliers(3000, 3, seed=24), 33),
    # the small-d seed keeps the 32 best in registers for k <= 32
    ("k32", lambda: synthetic.clusters_with_outliers(2500, 8, seed=32), 32),
    ("d1", lambda: synthetic.clusters_with_outliers(2000, 1, seed=25), 10),
    # the small-d seed covers tiles T, T+1, T-1, T+2, T-2: three to five
    # tiles leave the sweep nothing; six leave it one tile per row tile
    ("n300_seed_only", lambda: synthetic.clusters_with_outliers(300, 8, seed=29), 20),
    ("n385_k64", lambda: synthetic.clusters_with_outliers(385, 6, seed=30), 64),
    # the wide-point sweep: d not a multiple of 16, d = 128 with k = 50
    ("d9", lambda: synthetic.clusters_with_outliers(3000, 9, seed=26), 20),
    ("d100_k40", lambda: synthetic.reference_test_data(2500, 100, seed=27, n_outliers=25), 40),
    ("factor_d128_k50", lambda: synthetic.factor_model(3000, 128, seed=28), 50),
    # 10,000 points on 50 positions: every point has 199 exact duplicates,
    # which keeps the lists full of exact ties (and, on the tensor path,
    # drives rows into exact-key lists)
    ("dups_heavy", lambda: np.repeat(np.random.default_rng(5).uniform(-3, 3, (50, 4)).astype(np.float32), 200,
                                     axis=0)[np.random.default_rng(6).permutation(10_000)], 20),
]


@pytest.mark.parametrize("path", KNN_PATHS)
@pytest.mark.parametrize("name,make,k", KNN_CASES, ids=[c[0] for c in KNN_CASES])
def test_knn_bit_exact_vs_oracle(ctx, path, name, make, k):
    X = make()
    if path in (_culof.PATH_FAST, _culof.PATH_TENSOR) and (k > 64 or X.shape[1] > 128):
        pytest.skip("the fused paths take k <= 64 and d <= 128")
    ctx.set_path(path)
    idx, d2, kd = run_knn(ctx, X, k)
    Xc, _, _ = oracle.center(X)
    o_idx, o_d2, o_kd = oracle.knn(Xc, k)
    np.testing.assert_array_equal(kd.view(np.uint32), o_kd.view(np.uint32))
    np.testing.assert_array_equal(idx, o_idx)
    np.testing.assert_array_equal(d2.view(np.uint32), o_d2.view(np.uint32))


@pytest.mark.parametrize("name", ["clusters", "ragged", "k64", "n385_k64", "d1", "dups_heavy"])
def test_knn_without_prune_lists_bit_exact(ctx, monkeypatch, name):
    # inputs above 16,384 row tiles sweep the whole spiral without per-tile
    # candidate lists; CULOF_PRUNE_LISTS=0 takes that path at any size
    monkeypatch.setenv("CULOF_PRUNE_LISTS", "0")
    make, k = {c[0]: (c[1], c[2]) for c in KNN_CASES}[name]
    X = make()
    ctx.set_path(_culof.PATH_FAST)
    idx, d2, kd = run_knn(ctx, X, k)
    Xc, _, _ = oracle.center(X)
    o_idx, o_d2, o_kd = oracle.knn(Xc, k)
    np.testing.assert_array_equal(kd.view(np.uint32), o_kd.view(np.uint32))
    np.testing.assert_array_equal(idx, o_idx)
    np.testing.assert_array_equal(d2.view(np.uint32), o_d2.view(np.uint32))


ISO_CASES = ["clusters", "clusters_k1", "lowdim", "d5_k25", "ragged", "dups", "k64", "k33_d3", "k32", "d1",
             "dups_heavy"]


@pytest.mark.parametrize("lists", ["1", "0"])
@pytest.mark.parametrize("name", ISO_CASES)
def test_knn_with_isolated_rows_bit_exact(ctx, monkeypatch, name, lists):
    # the rows with the largest seed k-th keys (about 1.2%) leave the small-d
    # sweep for their own pass from 16,384 points on; CULOF_ISO_ROWS=1 takes
    # that path at any size, with and without the per-tile candidate lists
    monkeypatch.setenv("CULOF_ISO_ROWS", "1")
    monkeypatch.setenv("CULOF_PRUNE_LISTS", lists)
    make, k = {c[0]: (c[1], c[2]) for c in KNN_CASES}[name]
    X = make()
    ctx.set_path(_culof.PATH_FAST)
    idx, d2, kd = run_knn(ctx, X, k)
    Xc, _, _ = oracle.center(X)
    o_idx, o_d2, o_kd = oracle.knn(Xc, k)
    np.testing.assert_array_equal(kd.view(np.uint32), o_kd.view(np.uint32))
    np.testing.assert_array_equal(idx, o_idx)
    np.testing.assert_array_equal(d2.view(np.uint32), o_d2.view(np.uint32))


@pytest.mark.parametrize("iso", ["0", "1"])
@pytest.mark.parametrize("k", [20, 40])
def test_isolated_rows_do_not_change_lof(ctx, monkeypatch, iso, k):
    # 30,000 points: 235 row tiles and isolated rows in most of them
    monkeypatch.setenv("CULOF_ISO_ROWS", iso)
    X = synthetic.clusters_with_outliers(30_000, 8, seed=41)
    ctx.set_path(_culof.PATH_FAST)
    got = ctx.lof(X, k)
    np.testing.assert_array_equal(got.view(np.uint32), oracle.lof(X, k).view(np.uint32))


def test_results_are_ordered_on_the_callers_stream(ctx):
    # the small-d path forks its sweep and the isolated rows' pass onto two
    # internal streams and joins them back: a copy queued on the caller's
    # stream right after the call (no synchronisation in between) sees the
    # complete results, call after call
    torch = torch_cuda()
    X = synthetic.clusters_with_outliers(30_000, 8, seed=43)
    n, d, k = X.shape[0], X.shape[1], 20
    Xc, _, _ = oracle.center(X)
    o_idx, o_d2, o_kd = oracle.knn(Xc, k)
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    with torch.cuda.stream(s):
        dx = torch.from_numpy(X).to("cuda", non_blocking=False)
        for _ in range(3):
            idx = torch.full((k, n), -1, dtype=torch.int32, device="cuda")
            d2 = torch.full((k, n), float("nan"), dtype=torch.float32, device="cuda")
            kd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
            ctx.knn_device(dx.data_ptr(), n, d, k, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
            h_idx, h_d2, h_kd = (t.to("cpu", non_blocking=True) for t in (idx, d2, kd))
            s.synchronize()
            np.testing.assert_array_equal(h_idx.numpy(), o_idx)
            np.testing.assert_array_equal(h_d2.numpy().view(np.uint32), o_d2.view(np.uint32))
            np.testing.assert_array_equal(h_kd.numpy().view(np.uint32), o_kd.view(np.uint32))


def test_auto_selects_the_fast_path_for_small_d(ctx):
    X = synthetic.clusters_with_outliers(6000, 8, seed=1)
    ctx.lof(X, 20)
    assert ctx.last_path() == _culof.PATH_FAST
    # d <= 8 takes the FP32 sweep at every k the fused paths take (128-key
    # lists for k > 48)
    ctx.lof(X, 64)
    assert ctx.last_path() == _culof.PATH_FAST
    # up to 4096 points the general path's few kernels beat the fused paths
    ctx.lof(synthetic.clusters_with_outliers(3000, 8, seed=1), 20)
    assert ctx.last_path() == _culof.PATH_GENERAL
    ctx.lof(synthetic.reference_test_data(600, 4, seed=5), 257)
    assert ctx.last_path() == _culof.PATH_GENERAL
    ctx.lof(synthetic.reference_test_data(6000, 32, seed=5), 20)
    assert ctx.last_path() == _culof.PATH_TENSOR
    # 8 < d <= 16: the FP32 wide sweep below one wave of tensor CTAs, else the tensor path
    ctx.lof(synthetic.reference_test_data(6000, 12, seed=5), 20)
    assert ctx.last_path() == _culof.PATH_FAST
    ctx.lof(synthetic.clusters_with_outliers(40_000, 16, seed=5), 20)
    assert ctx.last_path() == _culof.PATH_TENSOR
    ctx.lof(synthetic.reference_test_data(600, 200, seed=5), 20)
    assert ctx.last_path() == _culof.PATH_GENERAL


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("normalize", [False, True])
def test_scores_bit_exact_vs_oracle(ctx, path, normalize):
    X = synthetic.clusters_with_outliers(5000, 8, seed=5)
    X[:, 3] *= 40.0
    ctx.set_path(path)
    got = ctx.lof(X, 20, normalize)
    want = oracle.lof(X, 20, normalize)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_constant_feature_with_normalize(ctx):
    rng = np.random.default_rng(6)
    X = rng.standard_normal((500, 3)).astype(np.float32)
    X[:, 1] = 7.0
    got = ctx.lof(X, 20, True)
    assert np.isfinite(got).all()
    np.testing.assert_array_equal(got, oracle.lof(X, 20, True))


@pytest.mark.parametrize("contamination", ["auto", 0.001, 0.01, 0.0123, 0.1, 0.5])
def test_fit_predict_bit_exact_vs_oracle(ctx, contamination):
    X = synthetic.clusters_with_outliers(6000, 8, seed=9)
    nof, labels, off = ctx.fit_predict(X, 20, False, contamination)
    o_labels, o_nof, o_off = oracle.fit_predict(X, 20, contamination)
    np.testing.assert_array_equal(nof, o_nof)
    assert off == o_off
    np.testing.assert_array_equal(labels, o_labels)


def test_offset_and_labels_match_reference_python_layer(ctx, ref_layer_golden):
    torch = torch_cuda()
    for case in ref_layer_golden.meta["cases"]:
        scores = ref_layer_golden[f"{case['scores']}/scores"]
        nof = dev(-scores)
        off = torch.zeros(1, dtype=torch.float64, device="cuda")
        ctx.offset_device(nof.data_ptr(), case["n"], case["contamination"], off.data_ptr())
        ctx.synchronize()
        assert float(off.item()) == case["offset"], case


@pytest.mark.parametrize("rows,row_offset,k", [(40, 100, 17), (1, 0, 1), (300, 0, 299), (7, 293, 64)])
def test_select_knn_tile_bit_exact_with_injected_distances(rows, row_offset, k):
    """The reference's select contract (culof_internal.cuh:37-53) fed exact
    distances: norms 0 and tile = -d2/2 make raw = d2 exactly."""
    torch = torch_cuda()
    rng = np.random.default_rng(rows + k)
    n = 300
    D = np.abs(rng.standard_normal((rows, n))).astype(np.float32) ** 3
    D[:, ::5] = D[:, 2:3]  # exact ties at many columns
    D[:, 7] = 0.0
    tile_np = (-D / 2).astype(np.float32)
    tile = dev(tile_np)
    norms = torch.zeros(n, dtype=torch.float32, device="cuda")
    idx = torch.full((k, n), -1, dtype=torch.int32, device="cuda")
    d2 = torch.full((k, n), float("nan"), dtype=torch.float32, device="cuda")
    kd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    _culof.select_knn_tile(0, tile.data_ptr(), norms.data_ptr(), rows, row_offset, n, k, idx.data_ptr(),
                           d2.data_ptr(), kd.data_ptr())
    torch.cuda.synchronize()
    o_idx, o_d2, o_kd = oracle.ref_select_tile(tile_np, np.zeros(n, np.float32), row_offset, k)
    cols = slice(row_offset, row_offset + rows)
    np.testing.assert_array_equal(host(kd)[cols].view(np.uint32), o_kd[cols].view(np.uint32))
    np.testing.assert_array_equal(host(idx)[:, cols], o_idx[:, cols])
    np.testing.assert_array_equal(host(d2)[:, cols].view(np.uint32), o_d2[:, cols].view(np.uint32))
    # the tile was converted in place to distances, diagonal +inf (knn.cu:150-152)
    conv = host(tile)
    expect = D.copy()
    expect[np.arange(rows), row_offset + np.arange(rows)] = np.inf
    np.testing.assert_array_equal(conv, expect)


def test_select_knn_tile_on_a_gram_tile():
    """A real Gram tile (float32 GEMM) with real norms: identical to the CPU
    restatement of the reference's conversion and select."""
    torch = torch_cuda()
    X = synthetic.clusters_with_outliers(2000, 8, seed=12)
    Xc, _, _ = oracle.center(X)
    norms_np = oracle.norms(Xc)
    rows, row0, k = 64, 512, 20
    G = (Xc[row0:row0 + rows].astype(np.float64) @ Xc.T.astype(np.float64)).astype(np.float32)
    tile = dev(G)
    norms = dev(norms_np)
    n = X.shape[0]
    idx = torch.full((k, n), -1, dtype=torch.int32, device="cuda")
    d2 = torch.full((k, n), float("nan"), dtype=torch.float32, device="cuda")
    kd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    _culof.select_knn_tile(0, tile.data_ptr(), norms.data_ptr(), rows, row0, n, k, idx.data_ptr(), d2.data_ptr(),
                           kd.data_ptr())
    torch.cuda.synchronize()
    o_idx, o_d2, o_kd = oracle.ref_select_tile(G, norms_np, row0, k)
    cols = slice(row0, row0 + rows)
    np.testing.assert_array_equal(host(kd)[cols].view(np.uint32), o_kd[cols].view(np.uint32))
    np.testing.assert_array_equal(host(idx)[:, cols], o_idx[:, cols])


def test_lrd_and_score_stage_entry_points():
    torch = torch_cuda()
    X = synthetic.clusters_with_outliers(3000, 8, seed=8)
    Xc, _, _ = oracle.center(X)
    idx, d2, kd = oracle.knn(Xc, 20)
    n, k = X.shape[0], 20
    lrd = torch.empty(n, dtype=torch.float32, device="cuda")
    sc = torch.empty(n, dtype=torch.float32, device="cuda")
    didx, dd2, dkd = dev(idx), dev(d2), dev(kd)
    _culof.compute_lrd(0, didx.data_ptr(), dd2.data_ptr(), dkd.data_ptr(), n, k, lrd.data_ptr())
    _culof.compute_scores(0, didx.data_ptr(), lrd.data_ptr(), n, k, sc.data_ptr())
    torch.cuda.synchronize()
    o_lrd = oracle.lrd(idx, d2, kd)
    np.testing.assert_array_equal(host(lrd), o_lrd)
    np.testing.assert_array_equal(host(sc), oracle.score(idx, o_lrd))


@pytest.mark.parametrize("n,swept", [(20_000, True), (300, False)])
def test_pair_stats_cover_the_sweep_past_the_seed_window(ctx, n, swept):
    # the small-d seed covers tiles T and T+-1, T+-2; the sweep every later tile
    X = synthetic.clusters_with_outliers(n, 8, seed=31)
    ctx.set_path(_culof.PATH_FAST)
    ctx.lof(X, 20)
    ev, tot = ctx.pair_stats()
    nt = (n + 127) // 128
    if swept:
        assert tot == nt * (nt - 5) * 128 * 128
        assert 0 < ev <= tot
    else:
        assert ev == 0 and tot == 0


def test_repeated_calls_are_bit_identical(ctx):
    X = synthetic.reference_test_data(512, 6, seed=17, n_outliers=7)
    first = ctx.lof(X, 20)
    for _ in range(3):
        np.testing.assert_array_equal(first, ctx.lof(X, 20))


@pytest.mark.parametrize("rows", ["1", "7", "64", "699"])
def test_tiling_does_not_change_results(monkeypatch, rows):
    """test_culof.cu:168-183, but bit-exact: tile height changes nothing."""
    X = synthetic.reference_test_data(700, 5, seed=13, n_outliers=9)
    monkeypatch.delenv("CULOF_TILE_ROWS", raising=False)
    with _culof.Context() as c:
        c.set_path(_culof.PATH_GENERAL)
        whole = c.lof(X, 25)
        monkeypatch.setenv("CULOF_TILE_ROWS", rows)
        np.testing.assert_array_equal(whole, c.lof(X, 25))


GOLDEN = golden_case_arrays()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_golden_scores_vs_sklearn(ctx, name, sk_golden):
    """The engine against scikit-learn fixtures (test_parity.py:20-67, REL_TOL
    2e-4), and bit-exact with the oracle."""
    X, k, normalize = GOLDEN[name]
    got = ctx.lof(X, k, normalize)
    np.testing.assert_array_equal(got, oracle.lof(X, k, normalize))
    want = sk_golden[f"{name}/scores"]
    rel = rel_err(got, want)
    if name == "duplicates":
        assert np.max(np.abs(got - want)) < 1e-2
        return
    bad = np.flatnonzero(rel >= 2e-4)
    if len(bad):
        gap = (sk_golden[f"{name}/dist_k1"] - sk_golden[f"{name}/dist_k"]) / np.maximum(sk_golden[f"{name}/dist_k"],
                                                                                           1e-12)
        assert gap[bad].max() < 1e-3
    if X.shape[0] >= 20_000:
        assert np.median(rel) < 1e-6 and np.percentile(rel, 99) < 1e-5
        nof, labels, _ = ctx.fit_predict(X, k, normalize, 0.01)
        want_out = np.unpackbits(sk_golden[f"{name}/outlier_bits"])[: X.shape[0]].astype(bool)
        assert np.array_equal(labels == -1, want_out)

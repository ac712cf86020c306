"""GPU parity: the GB300 learner against the oracle on identical seeded inputs.

* quantized path: split records, leaf values, root outputs and the partition are compared
  bit for bit (integer histograms are exact, so the trees must be identical);
* float path: the tree structure must match and every split gain must agree to 1e-6 relative;
  near-tie divergences are counted and reported;
* the reference's golden models are rebuilt through the GPU learner.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _skip_without_gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    _skip_without_gpu()


def _dataset(n, F, seed, nan_frac=0.1, int_frac=0.3, max_bin=255, zero_as_missing=False, min_data_in_leaf=20,
             feature_pre_filter=True):
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, F)).astype(np.float64)
    ni = int(F * int_frac)
    X[:, :ni] = rng.integers(0, 16, size=(n, ni))
    if nan_frac:
        X[rng.random((n, F)) < nan_frac] = np.nan
    w = rng.standard_normal(F)
    z = np.nan_to_num(X) @ w * 0.3 + np.sin(np.nan_to_num(X[:, -1]))
    ds = BinnedDataset.from_dense(X, max_bin=max_bin, zero_as_missing=zero_as_missing,
                                  min_data_in_leaf=min_data_in_leaf, feature_pre_filter=feature_pre_filter)
    return ds, z


def _grads(z, kind, seed):
    rng = np.random.default_rng(seed)
    n = len(z)
    if kind == "l2":
        y = z + rng.normal(0, 0.3, n)
        score = rng.normal(0, 0.1, n)
        return (score - y).astype(np.float32), np.ones(n, np.float32), True
    p = 1.0 / (1.0 + np.exp(-z))
    y = rng.random(n) < p
    score = rng.normal(0, 0.5, n)
    prob = 1.0 / (1.0 + np.exp(-score))
    g = (prob - y).astype(np.float32)
    h = (prob * (1.0 - prob)).astype(np.float32)
    return g, h, False


def _learners(ds, const_hess, loop_mode=1, num_jobs=1, **cfg):
    import harness
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig
    c = LearnerConfig(**cfg, is_constant_hessian=int(const_hess))
    return harness.OracleLearner(ds, c), GpuTreeLearner(ds, c, num_jobs=num_jobs, loop_mode=loop_mode), c


def _assert_records_equal(a, b):
    assert len(a) == len(b), "number of splits %d != %d" % (len(a), len(b))
    for i, (x, y) in enumerate(zip(a, b)):
        for name in a.dtype.names:
            xv, yv = x[name], y[name]
            if isinstance(xv, np.ndarray):  # the categorical bin bitset
                same = np.array_equal(xv, yv)
            elif isinstance(xv, (np.floating, float)):
                same = (xv == yv) or (np.isnan(xv) and np.isnan(yv))
            else:
                same = xv == yv
            assert same, "split %d field %s: oracle %r gpu %r" % (i, name, xv, yv)


QUANT_CASES = [
    dict(num_leaves=31, stochastic_rounding=1, num_grad_quant_bins=4),
    dict(num_leaves=63, stochastic_rounding=0, num_grad_quant_bins=4, lambda_l2=1.0),
    dict(num_leaves=15, stochastic_rounding=1, num_grad_quant_bins=16, lambda_l1=0.5, min_data_in_leaf=5),
    dict(num_leaves=31, stochastic_rounding=1, num_grad_quant_bins=6, max_delta_step=0.7, path_smooth=2.0),
    dict(num_leaves=31, stochastic_rounding=1, num_grad_quant_bins=4, quant_train_renew_leaf=1, max_depth=5),
    # 64 gradient bins: a 16:16 counter could overflow within one round of rows, so the histogram
    # kernel takes its wide form (32-bit gradient and hessian counters, no hot counters)
    dict(num_leaves=31, stochastic_rounding=1, num_grad_quant_bins=64),
]


@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("kind", ["binary", "l2"])
@pytest.mark.parametrize("case", range(len(QUANT_CASES)))
def test_quantized_trees_bit_exact(case, kind, fused):
    cfg = dict(QUANT_CASES[case], use_quantized_grad=1, seed=7, num_threads=4, fused_madd=fused)
    ds, z = _dataset(30000, 24, seed=case)
    g, h, const = _grads(z, kind, seed=case + 10)
    orc, gpu, c = _learners(ds, const, **cfg)
    rng = np.random.default_rng(1)
    for it in range(3):
        ro = orc.train(g, h)
        rg = gpu.train(g, h)
        _assert_records_equal(ro[0], rg[0])
        assert np.array_equal(ro[1], rg[1]), "leaf values differ at tree %d" % it
        assert ro[2] == rg[2]
        assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
        g = (g + rng.normal(0, 0.05, len(g))).astype(np.float32)
    gpu.close()


def test_quantized_bagged_rows_and_zero_missing():
    cfg = dict(num_leaves=31, use_quantized_grad=1, stochastic_rounding=1, seed=3, num_threads=2)
    ds, z = _dataset(20000, 16, seed=5, zero_as_missing=True, nan_frac=0.0)
    g, h, const = _grads(z, "binary", seed=6)
    orc, gpu, _ = _learners(ds, const, **cfg)
    rows = np.sort(np.random.default_rng(2).choice(ds.num_data, 12000, replace=False)).astype(np.int32)
    for rr in (rows, None, rows):
        ro = orc.train(g, h, rr)
        rg = gpu.train(g, h, rr)
        _assert_records_equal(ro[0], rg[0])
        assert np.array_equal(ro[1], rg[1])
        assert np.array_equal(orc.row_leaf(), gpu.row_leaf())


def test_loop_modes_agree():
    cfg = dict(num_leaves=63, use_quantized_grad=1, stochastic_rounding=0)
    ds, z = _dataset(20000, 40, seed=9)
    g, h, const = _grads(z, "binary", seed=1)
    _, gpu0, c = _learners(ds, const, loop_mode=0, **cfg)
    from lgbm_gb300 import GpuTreeLearner
    gpu1 = GpuTreeLearner(ds, c, loop_mode=1)
    a, b = gpu0.train(g, h), gpu1.train(g, h)
    _assert_records_equal(a[0], b[0])
    assert np.array_equal(a[1], b[1])


def test_multiclass_jobs_batched_match_sequential_oracle():
    """K class trees grown in one call equal K sequential oracle trees (one shared discretizer)."""
    K = 3
    cfg = dict(num_leaves=15, use_quantized_grad=1, stochastic_rounding=1, seed=11, num_threads=3)
    ds, z = _dataset(15000, 20, seed=4)
    rng = np.random.default_rng(0)
    G = rng.normal(0, 1, (K, ds.num_data)).astype(np.float32)
    H = rng.uniform(0.05, 0.25, (K, ds.num_data)).astype(np.float32)
    orc, gpu, _ = _learners(ds, False, num_jobs=K, **cfg)
    for it in range(2):
        splits, lv, roots, nls = gpu.train_raw(G, H)
        rl = gpu.row_leaf()
        for k in range(K):
            ro = orc.train(G[k], H[k])
            _assert_records_equal(ro[0], splits[k, :nls[k] - 1])
            assert np.array_equal(ro[1], lv[k, :nls[k]])
            assert np.array_equal(orc.row_leaf(), rl[k])
        G = (G * 0.9).astype(np.float32)


@pytest.mark.parametrize("quant", [1, 0])
def test_feature_mask_per_job(quant):
    """bk_learner_set_feature_mask: one by-tree column sample per class tree (serial.rs:839-854);
    the quantized trees equal the oracle's bit for bit, the float trees within tolerance."""
    K = 3
    cfg = dict(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=5, num_threads=2)
    ds, z = _dataset(20000, 24, seed=8)
    rng = np.random.default_rng(3)
    G = rng.normal(0, 1, (K, ds.num_data)).astype(np.float32)
    H = rng.uniform(0.05, 0.25, (K, ds.num_data)).astype(np.float32)
    orc, gpu, _ = _learners(ds, False, num_jobs=K, **cfg)
    divergences = []
    for it in range(3):
        mask = rng.random((K, ds.num_features)) < 0.5
        mask[:, it] = True  # at least one feature per tree
        gpu.set_feature_mask(mask)
        splits, lv, roots, nls = gpu.train_raw(G, H)
        rl = gpu.row_leaf()
        for k in range(K):
            used = set(np.flatnonzero(mask[k]).tolist())
            assert set(splits[k, :nls[k] - 1]["inner_feature"].tolist()) <= used
            orc.set_feature_mask(mask[k])
            ro = orc.train(G[k], H[k])
            if quant:
                _assert_records_equal(ro[0], splits[k, :nls[k] - 1])
                assert np.array_equal(ro[1], lv[k, :nls[k]])
                assert np.array_equal(orc.row_leaf(), rl[k])
            else:
                rg = (splits[k, :nls[k] - 1], lv[k, :nls[k]], roots[k])
                d = _float_compare(ro, rg)
                if d >= 0:
                    divergences.append((it, k, d))
    # float near-tie split choices are allowed but must be rare
    print("float near-tie divergences (call, job, split):", divergences)
    assert len(divergences) <= 1
    # the mask stays until it is replaced; None restores every feature
    gpu.set_feature_mask(None)
    orc.set_feature_mask(None)
    splits, lv, roots, nls = gpu.train_raw(G, H)
    ro = orc.train(G[0], H[0])
    if quant:
        _assert_records_equal(ro[0], splits[0, :nls[0] - 1])
    gpu.close()


def _float_compare(ro, rg):
    """Structure equal, gains within 1e-6 relative; returns the index of the first near-tie
    divergence (or -1)."""
    a, b = ro[0], rg[0]
    n = min(len(a), len(b))
    for i in range(n):
        same = all(a[i][k] == b[i][k] for k in ("leaf", "real_feature", "threshold", "default_left",
                                                  "left_count", "right_count"))
        if not same:
            return i
        ga, gb = float(a[i]["gain"]), float(b[i]["gain"])
        assert abs(ga - gb) <= 1e-6 * max(abs(ga), 1e-300), "split %d gain %r vs %r" % (i, ga, gb)
        for k in ("left_output", "right_output", "left_sum_gradient", "right_sum_gradient", "left_sum_hessian",
                  "right_sum_hessian"):
            x, y = float(a[i][k]), float(b[i][k])
            assert abs(x - y) <= 1e-6 * max(abs(x), 1e-9) + 1e-9, "split %d %s %r vs %r" % (i, k, x, y)
    return -1 if len(a) == len(b) else n


@pytest.mark.parametrize("kind", ["l2", "binary"])
@pytest.mark.parametrize("extra", [dict(), dict(lambda_l1=0.3, lambda_l2=2.0, min_gain_to_split=0.01),
                                   dict(max_delta_step=0.5, path_smooth=3.0)])
def test_float_trees_match(kind, extra):
    cfg = dict(num_leaves=63, **extra)
    ds, z = _dataset(40000, 30, seed=2)
    g, h, const = _grads(z, kind, seed=3)
    orc, gpu, _ = _learners(ds, const, **cfg)
    divergences = []
    for it in range(3):
        ro, rg = orc.train(g, h), gpu.train(g, h)
        d = _float_compare(ro, rg)
        if d >= 0:
            divergences.append((it, d))
        g = (g * 0.8).astype(np.float32)
    # near-tie split choices are allowed but must be rare; report them
    print("float near-tie divergences (tree, split):", divergences)
    assert len(divergences) <= 1


CASES = sorted(os.listdir(os.path.join(GOLDEN, "train")))


@pytest.mark.parametrize("case", CASES)
def test_gpu_reproduces_reference_models(oracle, case):
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    d = os.path.join(GOLDEN, "train", case)
    P = json.load(open(os.path.join(d, "params.json")))
    p = P["params"]
    X = np.load(os.path.join(d, "x.npy"))
    y = np.load(os.path.join(d, "y.npy"))
    wp = os.path.join(d, "w.npy")
    weights = np.load(wp) if os.path.exists(wp) else None
    ds = BinnedDataset.from_dense(X, max_bin=p.get("max_bin", 255), min_data_in_leaf=p.get("min_data_in_leaf", 20),
                                  zero_as_missing=p.get("zero_as_missing", False),
                                  categorical=P.get("categorical", []))
    obj = oracle.make_objective(p, y, weights, fused=True)
    cfg = LearnerConfig(**p, fused_madd=1, is_constant_hessian=int(obj.constant_hessian and
                                                                       p.get("data_sample_strategy") != "goss"))
    learner = GpuTreeLearner(ds, cfg)
    model = open(os.path.join(d, "model.txt")).read()
    cols, bag = oracle.samplers_from_params(oracle.resolved_params(model), ds)
    trees, _ = oracle.train_gbdt(learner, ds, obj, P["num_boost_round"], learning_rate=p.get("learning_rate", 0.1),
                                 boost_from_average=p.get("boost_from_average", True),
                                 min_gain_to_split=p.get("min_gain_to_split", 0.0), col_sampler=cols, bagging=bag)
    ref = oracle.parse_model_trees(model)
    assert len(trees) == len(ref)
    for i, (t, r) in enumerate(zip(trees, ref)):
        bad = oracle.compare_tree(t, r, leaf_rtol=1e-9)
        assert not bad, "tree %d differs in %s" % (i, bad)


def test_tiny_leaf_counts_give_a_stump():
    """Fewer rows than 2 * min_data_in_leaf: no split (serial.rs:795-803)."""
    ds, z = _dataset(30, 4, seed=1, nan_frac=0.0, feature_pre_filter=False)
    g, h, const = _grads(z, "l2", seed=2)
    orc, gpu, _ = _learners(ds, const, num_leaves=7, min_data_in_leaf=20)
    ro, rg = orc.train(g, h), gpu.train(g, h)
    assert len(ro[0]) == len(rg[0]) == 0
    assert ro[2] == rg[2]


def test_device_prediction_replays_the_partition():
    """bk_learner_predict_add on the training rows' bins lands every row in the leaf the
    partition put it in (serial.rs:2009-2041 replays splits with the training routing)."""
    import torch
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig, Tree
    ds, z = _dataset(20000, 20, seed=12, zero_as_missing=False)
    g, h, const = _grads(z, "binary", seed=13)
    for quant in (1, 0):
        cfg = LearnerConfig(num_leaves=31, use_quantized_grad=quant, is_constant_hessian=int(const))
        gpu = GpuTreeLearner(ds, cfg)
        splits, lv, root = gpu.train(g, h)
        t = Tree.from_records(31, splits, lv, root, ds.features)
        row_leaf = gpu.row_leaf()
        bins = torch.from_numpy(np.ascontiguousarray(ds.bins)).cuda()
        score = torch.zeros(ds.num_data, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        gpu.predict_add(t, bins.data_ptr(), ds.num_data, score.data_ptr())
        got = score.cpu().numpy()
        assert np.array_equal(got, t.leaf_value[row_leaf])
        gpu.close()


@pytest.mark.parametrize("shape", [(32, 1, 1, 0), (64, 3, 7, 0), (1024, 200, 1024, 0), (256, 38, 304, 0),
                                   (64, 3, 7, 1 << 30), (256, 38, 304, 512), (32, 64, 64, 96),
                                   (256, 38, 304, 0, 2), (256, 38, 304, 0, 4), (64, 9, 33, 0, 4),
                                   (32, 2, 8, 0, 8), (256, 38, 304, 512, 4)])
def test_launch_shapes_do_not_change_results(shape):
    """Every launch shape grows the oracle's trees: quantized bit-exact, both partition forms,
    with the shared-histogram CTAs, the global-atomic CTAs (every CTA at 1 << 30) or a mix, and
    with clusters of 2, 4 or 8 histogram CTAs adding up their histograms in distributed shared
    memory (leaves smaller than a cluster included: its CTAs without rows add zeros)."""
    cfg = dict(num_leaves=31, use_quantized_grad=1, stochastic_rounding=1, seed=2, num_threads=2)
    ds, z = _dataset(25000, 40, seed=21)
    g, h, const = _grads(z, "binary", seed=22)
    for loop_mode in (1, 0):
        orc, gpu, _ = _learners(ds, const, loop_mode=loop_mode, **cfg)
        gpu.set_launch_shape(shape)
        got = gpu.launch_shape()
        cl = shape[4] if len(shape) > 4 else 0
        assert got[4] == (1 if cl < 2 else cl) and got[1] % got[4] == 0
        # the tile's CTAs: at most the asked number, rounded to whole clusters (at least one)
        assert got[0] == max(32, shape[0] // 32 * 32) and 1 <= got[1] <= max(shape[1], got[4])
        assert 1 <= got[2] <= shape[2] and got[3] == shape[3]
        for it in range(2):
            ro, rg = orc.train(g, h), gpu.train(g, h)
            _assert_records_equal(ro[0], rg[0])
            assert np.array_equal(ro[1], rg[1])
            assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
            g = (g * 0.9).astype(np.float32)
        gpu.close()


def test_autotune_keeps_parity_and_caches_by_shape():
    """bk_learner_autotune times trial trees and restores the learner's state: the trees after it
    equal the oracle's (which never grew the trial trees); a second learner of the same shape
    class takes the cached shape."""
    cfg = dict(num_leaves=31, use_quantized_grad=1, stochastic_rounding=1, seed=4, num_threads=2)
    ds, z = _dataset(30000, 36, seed=23)
    g, h, const = _grads(z, "l2", seed=24)
    orc, gpu, c = _learners(ds, const, **cfg)
    shape = gpu.autotune(g, h, trials=1)
    assert shape == gpu.launch_shape()
    for it in range(2):
        ro, rg = orc.train(g, h), gpu.train(g, h)
        _assert_records_equal(ro[0], rg[0])
        assert np.array_equal(ro[1], rg[1])
        assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
        g = (g * 0.9).astype(np.float32)
    from lgbm_gb300 import GpuTreeLearner
    other = GpuTreeLearner(ds, c)
    assert other.autotune(g, h, trials=1) == shape
    gpu.close()
    other.close()


def _cat_dataset(n, seed, nan_frac=0.05):
    """Two categorical columns with 3 and 40 categories (one-hot and sorted searches), one with
    200 categories, plus numerical columns; the target depends on category groups."""
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 8))
    X[:, 0] = rng.integers(0, 3, n)
    X[:, 3] = rng.integers(0, 40, n)
    X[:, 6] = rng.integers(0, 200, n)
    X[rng.random((n, 8)) < nan_frac] = np.nan
    eff = rng.standard_normal(200)
    c3 = np.nan_to_num(X[:, 3], nan=0).astype(int)
    c6 = np.nan_to_num(X[:, 6], nan=0).astype(int)
    z = eff[c3 % 40] + 0.5 * eff[c6] + np.nan_to_num(X[:, 1]) + (np.nan_to_num(X[:, 0]) == 1)
    ds = BinnedDataset.from_dense(X, categorical=[0, 3, 6])
    assert sum(f.categorical for f in ds.features) == 3
    return ds, z


CAT_CASES = [dict(), dict(max_cat_to_onehot=64, min_data_per_group=20),
             dict(cat_smooth=2.0, cat_l2=1.0, max_cat_threshold=8, min_data_per_group=30, lambda_l2=0.5),
             dict(lambda_l1=0.2, max_delta_step=0.8, path_smooth=1.5, min_data_per_group=10)]


@pytest.mark.parametrize("case", range(len(CAT_CASES)))
def test_categorical_trees(case):
    """Categorical features (one-hot and sorted searches, bitset partitions): quantized trees
    bit-exact with the oracle's, float trees within the float tolerance."""
    ds, z = _cat_dataset(30000, seed=40 + case)
    for quant in (1, 0):
        for kind in ("binary", "l2"):
            g, h, const = _grads(z, kind, seed=50 + case)
            cfg = dict(CAT_CASES[case], num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=3,
                       num_threads=2)
            orc, gpu, _ = _learners(ds, const, **cfg)
            divergences = []
            ncat = 0
            for it in range(2):
                ro, rg = orc.train(g, h), gpu.train(g, h)
                ncat += int(np.sum(rg[0]["categorical"]))
                if quant:
                    _assert_records_equal(ro[0], rg[0])
                    assert np.array_equal(ro[1], rg[1])
                    assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
                else:
                    d = _float_compare(ro, rg)
                    if d >= 0:
                        divergences.append((it, d))
                    else:
                        assert all(np.array_equal(a["cat_bins"], b["cat_bins"]) for a, b in zip(ro[0], rg[0]))
                g = (g * 0.9).astype(np.float32)
            assert ncat > 0, "no categorical split was chosen"
            print("float near-tie divergences:", divergences)
            assert len(divergences) <= 1
            gpu.close()


@pytest.mark.parametrize("bytree,bynode,constrained", [(False, 0.35, False), (True, 0.35, False),
                                                       (False, 1.0, True), (True, 0.5, True)])
def test_bynode_column_sample(bytree, bynode, constrained):
    """bk_learner_set_bynode / bk_learner_set_interaction_constraints: every searched leaf gets its
    feature mask on the device (a sample from the sampler's LCG stream, the features its path's
    interaction constraints allow, or both); trees (quantized, bit-exact) and the stream's state
    after each tree equal the oracle's."""
    import harness
    ds, z = _dataset(20000, 60, seed=31)
    g, h, const = _grads(z, "binary", seed=32)
    cfg = dict(num_leaves=31, use_quantized_grad=1, stochastic_rounding=1, seed=5, num_threads=2)
    orc, gpu, _ = _learners(ds, const, **cfg)
    icons = [list(range(0, 20)), list(range(10, 35)), [40, 41, 42, 43, 59]] if constrained else None
    cols_o = harness.TreeColumnSampler(ds.num_features, 0.7 if bytree else 1.0, 9, bynode, icons)
    cols_g = harness.TreeColumnSampler(ds.num_features, 0.7 if bytree else 1.0, 9, bynode, icons)
    for it in range(3):
        cols_o.before_tree(orc)
        cols_g.before_tree(gpu)
        ro, rg = orc.train(g, h), gpu.train(g, h)
        cols_o.after_tree(orc)
        cols_g.after_tree(gpu)
        _assert_records_equal(ro[0], rg[0])
        assert np.array_equal(ro[1], rg[1])
        assert cols_o.rand.x == cols_g.rand.x, "sampler state after tree %d" % it
        g = (g * 0.9).astype(np.float32)
    gpu.set_bynode(1.0, False, 0)
    gpu.close()


@pytest.mark.parametrize("quant,grad_bins", [(1, 4), (1, 64), (0, 4)])
def test_packed_bin_tiles(quant, grad_bins):
    """Stored-bin tiles of every layout in one dataset: 32 features of at most 16 group bins (a
    4-bit tile, two bins per byte as io/bin_data.rs:20-30 stores them), 32 features of 8-bit bins
    and a last tile of 8 features (a 16-byte 8-bit run): the quantized trees equal the oracle's bit
    for bit, with shared-histogram and global-atomic histogram CTAs, in the histogram kernel's
    16:16 form (4 gradient bins) and its wide form (64); the float trees agree within the float
    tolerance."""
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(31)
    n, F = 40000, 72
    X = rng.standard_normal((n, F))
    X[:, 40:50] = rng.integers(0, 6, size=(n, 10))
    X[rng.random((n, F)) < 0.03] = np.nan
    z = np.nan_to_num(X) @ rng.standard_normal(F) * 0.3
    ds = BinnedDataset.from_dense(X, max_bin_by_feature=[15] * 32 + [255] * 40)
    gb = [fi.group_bins for fi in ds.features]
    assert len(gb) == F and max(gb[:32]) <= 16 and max(gb[32:64]) > 16
    g, h, const = _grads(z, "binary", seed=32)
    cfg = dict(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=3, num_threads=2,
               num_grad_quant_bins=grad_bins)
    shapes = [(256, 38, 304, 0), (64, 20, 64, 1 << 30), (128, 38, 64, 0, 4)] if quant else [(256, 38, 304, 0)]
    for shape in shapes:
        for loop_mode in (1, 0):
            orc, gpu, _ = _learners(ds, const, loop_mode=loop_mode, **cfg)
            gpu.set_launch_shape(shape)
            gg = g
            for it in range(2):
                ro, rg = orc.train(gg, h), gpu.train(gg, h)
                if quant:
                    _assert_records_equal(ro[0], rg[0])
                    assert np.array_equal(ro[1], rg[1])
                    assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
                else:
                    import harness
                    e = harness.gain_errors(rg[0], ro[0])
                    assert e["max_rel"] <= 1e-6, e
                gg = (gg * 0.9).astype(np.float32)
            gpu.close()


def test_pool_capacity_and_budget_reset():
    """histogram_cache_capacity reports the full pool (one slot per leaf); the budget-only reset of
    reset_histogram_pool_config (serial.rs:250-264) changes nothing: the next trees still equal
    the oracle's bit for bit."""
    cfg = dict(num_leaves=23, use_quantized_grad=1, stochastic_rounding=1, seed=4, num_threads=2)
    ds, z = _dataset(12000, 18, seed=51)
    g, h, const = _grads(z, "binary", seed=52)
    orc, gpu, _ = _learners(ds, const, **cfg)
    assert gpu.histogram_cache_capacity() == 23
    for it in range(2):
        ro, rg = orc.train(g, h), gpu.train(g, h)
        _assert_records_equal(ro[0], rg[0])
        assert np.array_equal(ro[1], rg[1])
        gpu.reset_histogram_pool_config()
        assert gpu.histogram_cache_capacity() == 23
        g = (g * 0.9).astype(np.float32)
    gpu.close()


@pytest.mark.parametrize("max_bin,nan_frac", [(15, 0.1), (31, 0.0), (63, 0.0)])
@pytest.mark.parametrize("quant", [1, 0])
def test_narrow_search_ctas(max_bin, nan_frac, quant):
    """Learners whose every feature has at most 63 searched bins run the single-pass search in
    64-thread CTAs (two warps per (leaf side, feature)): the quantized trees equal the oracle's bit
    for bit and the float trees agree within the float tolerance, as in the 256-thread form (the
    stepwise form, which keeps 256-thread CTAs, is checked beside it)."""
    import harness
    cfg = dict(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=6, num_threads=2)
    ds, z = _dataset(30000, 40, seed=61, max_bin=max_bin, nan_frac=nan_frac)
    assert max(fi.num_bin for fi in ds.features) <= 64
    g, h, const = _grads(z, "binary", seed=62)
    for loop_mode in (1, 0):
        orc, gpu, _ = _learners(ds, const, loop_mode=loop_mode, **cfg)
        assert gpu.search_threads() == (64 if loop_mode == 1 else 256)
        gg = g
        for it in range(3):
            ro, rg = orc.train(gg, h), gpu.train(gg, h)
            if quant:
                _assert_records_equal(ro[0], rg[0])
                assert np.array_equal(ro[1], rg[1])
                assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
            else:
                m = harness.split_match(rg[0], ro[0])
                assert m["max_rel"] <= 1e-6, m
                assert m["matched"] >= 0.8 * max(len(ro[0]), len(rg[0])), m
            gg = (gg * 0.9).astype(np.float32)
        gpu.close()

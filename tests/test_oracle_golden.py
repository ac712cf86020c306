"""Pins the oracle to the reference's own golden data (no GPU).

* the upstream-LightGBM models that bankai-lightgbm reproduces (tests/golden/train*/*), rebuilt
  tree by tree through the oracle learner, with both ``madd`` rounding modes (bagged cases pass
  their rows, feature-fraction cases a by-tree feature mask, drawn as the reference's Trainer
  draws them);
* the std::mt19937 / libc++ distribution vectors and the discretizer vectors;
* the upstream stumps of quantized_gradients.json;
* the reference's brute-force integer split search cases.
"""
import json
import math
import os
import platform
import sys

import numpy as np
import pytest

from conftest import GOLDEN

# train/: the cases the GPU learner is also checked on; train_oracle/: cases that differ only on
# the Trainer's side of the learner (binary objective options, bagging balanced by label)
CASES = ([("train", c) for c in sorted(os.listdir(os.path.join(GOLDEN, "train")))]
         + [("train_oracle", c) for c in sorted(os.listdir(os.path.join(GOLDEN, "train_oracle")))])


def _load_case(case, fused=1):
    d = os.path.join(GOLDEN, *case)
    P = json.load(open(os.path.join(d, "params.json")))
    X = np.load(os.path.join(d, "x.npy"))
    y = np.load(os.path.join(d, "y.npy"))
    wp = os.path.join(d, "w.npy")
    P["weights"] = np.load(wp) if os.path.exists(wp) else None
    model = open(os.path.join(d, _model_file(d, fused))).read()
    return P, X, y, model


# Models whose last bits depend on the platform's libm as well (cross_entropy_lambda's initial
# score takes log(expm1(mean))): on the darwin model their leaf values agree to 1e-12 relative.
LIBM_DEPENDENT = {"xentlambda"}


def _linux_x86_64():
    return sys.platform.startswith("linux") and platform.machine() == "x86_64"


def _model_file(d, fused):
    """The fixtures' model.txt comes from upstream's darwin/arm64 build, where the reference's
    ``madd`` is one fused multiply-add; for the cases whose model changes with that rounding the
    reference also keeps the model of its linux-x86_64 build (unfused madd, glibc's libm;
    crates/lgbm-core/tests/support/mod.rs:205-245), which the unfused mode is checked against."""
    if not fused and os.path.exists(os.path.join(d, "model.linux-x86_64.txt")) and _linux_x86_64():
        return "model.linux-x86_64.txt"
    return "model.txt"


def _bit_exact_expected(case, fused):
    d = os.path.join(GOLDEN, *case)
    if fused:
        return case[1] not in LIBM_DEPENDENT
    return _model_file(d, fused) != "model.txt"


def _dataset(p, X, categorical=()):
    from lgbm_gb300 import BinnedDataset
    return BinnedDataset.from_dense(X, max_bin=p.get("max_bin", 255), min_data_in_leaf=p.get("min_data_in_leaf", 20),
                                    zero_as_missing=p.get("zero_as_missing", False), categorical=categorical)


@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("case", CASES, ids=["/".join(c) for c in CASES])
def test_oracle_reproduces_reference_models(oracle, bklib, case, fused):
    from lgbm_gb300 import LearnerConfig
    P, X, y, model = _load_case(case, fused)
    p = P["params"]
    ds = _dataset(p, X, P.get("categorical", []))
    obj = oracle.make_objective(p, y, P["weights"], fused=bool(fused))
    cfg = LearnerConfig(**p, fused_madd=fused, is_constant_hessian=int(obj.constant_hessian and
                                                                       p.get("data_sample_strategy") != "goss"))
    learner = oracle.OracleLearner(ds, cfg)
    cols, bag = oracle.samplers_from_params(oracle.resolved_params(model), ds, y)
    if p.get("boosting") in ("rf", "random_forest"):
        trees = oracle.train_rf(learner, ds, obj, P["num_boost_round"], min_gain_to_split=p.get("min_gain_to_split", 0.0),
                                col_sampler=cols, bagging=bag)
    else:
        trees, _ = oracle.train_gbdt(learner, ds, obj, P["num_boost_round"], learning_rate=p.get("learning_rate", 0.1),
                                     boost_from_average=p.get("boost_from_average", True),
                                     min_gain_to_split=p.get("min_gain_to_split", 0.0), col_sampler=cols, bagging=bag)
    ref = oracle.parse_model_trees(model)
    assert len(trees) == len(ref)
    exact = total = 0
    for i, (t, r) in enumerate(zip(trees, ref)):
        bad = oracle.compare_tree(t, r)
        assert not bad, "tree %d differs in %s" % (i, bad)
        vals = np.array([float(v) for v in r["leaf_value"].split()])
        exact += int(np.sum(vals == t.leaf_value[:t.num_leaves]))
        total += t.num_leaves
    if _bit_exact_expected(case, fused):
        # fused mode against the FMA build's model, unfused mode against the linux-x86_64 model:
        # every leaf value bit-identical
        assert exact == total, "%d of %d leaf values bit-exact" % (exact, total)


def test_mt19937_standard_vector(oracle):
    v = json.load(open(os.path.join(GOLDEN, "vectors.json")))
    out = np.zeros(10000, dtype=np.uint64)
    oracle.load().orc_mt19937(5489, 0, 0, 10000, out.ctypes.data)
    assert int(out[-1]) == v["mt19937_default_10000th"]


def test_libcxx_distributions(oracle):
    v = json.load(open(os.path.join(GOLDEN, "vectors.json")))
    u = v["uniform_real_01"]
    out = np.zeros(len(u["bits"]), dtype=np.uint64)
    oracle.load().orc_mt19937(u["seed"], 1, 0, len(out), out.ctypes.data)
    assert [int(x) for x in out] == u["bits"]
    for case in v["uniform_int_inclusive"]:
        out = np.zeros(len(case["draws"]), dtype=np.uint64)
        oracle.load().orc_mt19937(case["seed"], 2, case["n"], len(out), out.ctypes.data)
        assert [int(x) for x in out] == case["draws"]


def _discretize(oracle, g, h, bins, const_hess, stochastic=0, seed=0, threads=1, fused=0, calls=1):
    g = np.asarray(g, np.float32)
    h = np.asarray(h, np.float32)
    out = np.zeros(len(g), np.int16)
    sc = np.zeros(2, np.float64)
    ok = oracle.load().orc_discretize(g.ctypes.data, h.ctypes.data, len(g), bins, const_hess, stochastic, seed,
                                      threads, fused, calls, out.ctypes.data, sc.ctypes.data)
    return ok, out, sc


def test_discretizer_vectors(oracle):
    v = json.load(open(os.path.join(GOLDEN, "vectors.json")))
    assert v["nearest_bins4"]
    for case in v["nearest_bins4"]:
        for fused in (0, 1):
            ok, out, sc = _discretize(oracle, case["gradients"], case["hessians"], 4, 0, fused=fused)
            assert ok
            assert out.tolist() == case["packed"]
            assert sc[0] == case["gradient_scale"] and sc[1] == case["hessian_scale"]
    c = v["nearest_const_hess_bins4"]
    ok, out, _ = _discretize(oracle, c["gradients"], c["hessians"], 4, 1)
    assert ok and out.tolist() == c["packed"]


def test_discretizer_refuses_degenerate_inputs(oracle):
    assert _discretize(oracle, [0.0, 0.0], [1.0, 1.0], 4, 0)[0] == 0
    assert _discretize(oracle, [1.0, 1.0], [-1.0, 1.0], 4, 0)[0] == 0
    assert _discretize(oracle, [np.nan, 1.0], [1.0, 1.0], 4, 0)[0] == 0


def test_quantized_gradient_stumps(oracle):
    """tests/fixtures/quantized_gradients.json: 16 upstream stumps (tolerance 1e-12 as the reference)."""
    d = json.load(open(os.path.join(GOLDEN, "quantized_gradients.json")))
    assert d["upstream"] == "4.7.0" and len(d["cases"]) == 16

    def close(a, b):
        assert abs(a - b) <= 1e-12 * max(abs(b), 1.0), (a, b)

    for c in d["cases"]:
        g = np.asarray(c["gradients"], np.float64).astype(np.float32)
        h = np.asarray(c["hessians"], np.float64).astype(np.float32)
        ok, packed, sc = _discretize(oracle, g, h, c["bins"], int(c["constant_hessian"]))
        assert ok
        left = np.zeros(len(g), bool)
        left[c["left_rows"]] = True
        gi = (packed >> 8).astype(np.int8).astype(np.int64)
        hi = (packed & 0xFF).astype(np.int64)
        lg, lh = gi[left].sum() * sc[0], hi[left].sum() * sc[1]
        rg, rh = gi[~left].sum() * sc[0], hi[~left].sum() * sc[1]
        close(lh, c["left_weight"])
        close(rh, c["right_weight"])
        close(-lg / lh, c["left_output"])
        close(-rg / rh, c["right_output"])
        gain = lg * lg / lh + rg * rg / rh - (lg + rg) ** 2 / (lh + rh)
        close(float(np.float32(gain)), c["split_gain"])


def _brute_force_int_split(hist, gs, hs, l2, min_data):
    """crates/lgbm-core/tests/quantized_split_search.rs:59-135, restated."""
    EPS = float(np.float32(1e-15))
    tg = sum(b[0] for b in hist)
    th = sum(b[1] for b in hist)
    num_data = th
    cnt_factor = num_data / float(th)

    def out(g, h):
        return -g / (h + l2)

    def gain_of(g, h):
        o = out(g, h)
        return -(2.0 * g * o + (h + l2) * o * o)

    mgs = gain_of(tg * gs, th * hs) + 0.0
    best = dict(splittable=False, gain=-math.inf)
    for s in range(1, len(hist)):
        rg = sum(b[0] for b in hist[s:])
        rh = sum(b[1] for b in hist[s:])
        lg, lh = tg - rg, th - rh
        rc = int(rh * cnt_factor + 0.5)
        lc = num_data - rc
        srh, slh = rh * hs, lh * hs
        if rc < min_data or lc < min_data:
            continue
        gain = gain_of(lg * gs, slh + EPS) + gain_of(rg * gs, srh + EPS)
        if gain <= mgs:
            continue
        best["splittable"] = True
        if gain > best["gain"]:
            best.update(gain=gain, threshold=s - 1, left_count=int(lh * cnt_factor + 0.5),
                        right_count=int(rh * cnt_factor + 0.5), left_output=out(lg * gs, slh),
                        right_output=out(rg * gs, srh))
    if best["splittable"]:
        best["gain"] -= mgs
    return best, tg, th, num_data


def test_int_split_search_brute_force(oracle):
    from lgbm_gb300 import LearnerConfig, FEATURE_DTYPE
    from lgbm_gb300.tree import SPLIT_DTYPE
    v = json.load(open(os.path.join(GOLDEN, "vectors.json")))
    assert v["int_split_search"]
    for case in v["int_split_search"]:
        hist = case["hist"]
        for gs, hs, l2, min_data in case["checks"]:
            want, tg, th, num_data = _brute_force_int_split(hist, gs, hs, l2, min_data)
            f = np.zeros(1, FEATURE_DTYPE)
            # offset 0 (the reference test's FeatureMeta): any nonzero most-frequent bin
            f[0] = (len(hist), 0, 0, 1, 1.0, 0, 0)
            cfg = LearnerConfig(lambda_l2=l2, min_data_in_leaf=min_data, min_sum_hessian_in_leaf=0.0).record()
            hg = np.array([b[0] for b in hist], np.int64)
            hh = np.array([b[1] for b in hist], np.int64)
            out = np.zeros(1, SPLIT_DTYPE)
            sp = oracle.load().orc_find_best_threshold_int(hg.ctypes.data, hh.ctypes.data, f.ctypes.data,
                                                            cfg.ctypes.data, tg, th, gs, hs, num_data, 0.0,
                                                            out.ctypes.data)
            assert bool(sp) == want["splittable"]
            if not want["splittable"]:
                continue
            o = out[0]
            assert o["threshold"] == want["threshold"]
            assert o["left_count"] == want["left_count"] and o["right_count"] == want["right_count"]
            assert abs(o["gain"] - want["gain"]) <= 1e-12 * max(abs(want["gain"]), 1.0)
            assert abs(o["left_output"] - want["left_output"]) <= 1e-12
            assert abs(o["right_output"] - want["right_output"]) <= 1e-12


@pytest.mark.parametrize("fused", [True, False])
def test_percentile_matches_order_statistics(oracle, fused):
    """The reference's unit check of its percentile (objective/regression.rs:487-503): between the
    order statistics around (n - 1) * (1 - alpha) counted from the largest, to 1e-12."""
    data = [5.0, 1.0, 4.0, 4.0, 2.0, 9.0, 7.0, 3.0]
    desc = sorted(data, reverse=True)
    for alpha in (0.1, 0.3, 0.5, 0.7, 0.9):
        got = oracle._percentile(data, alpha, False, fused)
        fp = (len(data) - 1) * (1.0 - alpha)
        pos = int(fp) + 1
        bias = fp - (pos - 1)
        v1, v2 = desc[pos - 1], desc[pos]
        assert abs(got - (v1 - (v1 - v2) * bias)) < 1e-12, alpha
    # with unit weights every step of the cumulative weight is 1, so the weighted form
    # interpolates between neighbouring order statistics too
    for alpha in (0.25, 0.5, 0.75):
        got = oracle._weighted_percentile(data, [1.0] * len(data), alpha, False, fused)
        assert min(data) <= got <= max(data)

"""ORACLE harness — test infrastructure only.

* ``OracleLearner``: ctypes wrapper over ``oracle/_build/liboracle.so`` (the C++ restatement of
  the reference's tree learner).
* A restatement of the reference's boosting loop around a learner
  (crates/lgbm-core/src/boosting/train.rs:723-839): objective gradients (binary
  objective/binary.rs:71-90, L2 objective/regression.rs:240-248, softmax
  objective/multiclass.rs:68-90), ``boost_from_average`` (train.rs:615-640), shrinkage and the
  score update (tree.rs:446-478, serial.rs:1974-1990).
* A parser for the tree sections of LightGBM model text, to compare against the reference's
  golden ``model.txt`` files.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use this module.
"""
import ctypes
import math
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "bankai-lightgbm_gb300"))

from lgbm_gb300.config import LearnerConfig  # noqa: E402
from lgbm_gb300.dataset import _Random as LcgRandom  # noqa: E402  (utils/random.rs, the bin sampler's LCG)
from lgbm_gb300.tree import SPLIT_DTYPE, Tree, _round_to_zero  # noqa: E402

EPS = float(np.float32(1e-15))
_olib = None


def load():
    global _olib
    if _olib is None:
        sys.path.insert(0, HERE)
        import build as obuild  # oracle/build.py
        path = obuild.build()
        lib = ctypes.CDLL(path)
        P, i32, i64, u32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32
        lib.orc_learner_create.restype = P
        lib.orc_learner_create.argtypes = [P, i32, P, i64, P]
        lib.orc_learner_destroy.argtypes = [P]
        lib.orc_learner_set_feature_mask.argtypes = [P, P]
        lib.orc_learner_set_bynode.argtypes = [P, ctypes.c_double, i32, u32]
        lib.orc_learner_bynode_state.restype = u32
        lib.orc_learner_bynode_state.argtypes = [P]
        lib.orc_learner_set_interaction_constraints.argtypes = [P, P, P, i32]
        lib.orc_learner_train.restype = i32
        lib.orc_learner_train.argtypes = [P, P, P, P, i64, P, P]
        lib.orc_learner_root_output.restype = ctypes.c_double
        lib.orc_learner_root_output.argtypes = [P]
        lib.orc_learner_row_leaf.argtypes = [P, P]
        lib.orc_learner_partition.argtypes = [P, P, P, P]
        lib.orc_learner_packed.argtypes = [P, P, P]
        lib.orc_hist_float.argtypes = [P, i64, i32, P, P, i64, P, P, i32, P]
        lib.orc_hist_int.argtypes = [P, i64, i32, P, P, i64, P, P, P]
        lib.orc_discretize.restype = i32
        lib.orc_discretize.argtypes = [P, P, i64, i32, i32, i32, u32, i32, i32, i32, P, P]
        lib.orc_mt19937.argtypes = [u32, i32, u32, i64, P]
        lib.orc_route_table.argtypes = [P, u32, i32, P]
        lib.orc_route_table_cat.argtypes = [P, P, P]
        lib.orc_find_best_threshold_int.restype = i32
        lib.orc_find_best_threshold_int.argtypes = [P, P, P, P, i64, i64, ctypes.c_double, ctypes.c_double, i32,
                                                    ctypes.c_double, P]
        lib.orc_find_best_threshold.restype = i32
        lib.orc_find_best_threshold.argtypes = [P, P, P, ctypes.c_double, ctypes.c_double, i32, ctypes.c_double, P]
        lib.orc_sizeof_split.restype = i32
        lib.orc_learner_set_threads.argtypes = [P, i32]
        lib.orc_learner_leaf_histogram.restype = i32
        lib.orc_learner_leaf_histogram.argtypes = [P, i32, P, P]
        lib.orc_learner_add_score.argtypes = [P, P, P]
        lib.orc_bin_dense_f32.restype = i32
        lib.orc_bin_dense_f32.argtypes = [P, i64, i32, i32, i32, i32, i64, i32, i32, i32, P, P, P, P]
        lib.orc_find_bin.restype = i32
        lib.orc_find_bin.argtypes = [P, i64, i64, i32, i32, i32, i32, i32, i32, P, i32, P, P]
        lib.orc_sample_rows.restype = i64
        lib.orc_sample_rows.argtypes = [i64, i64, i32, P]
        assert lib.orc_sizeof_split() == SPLIT_DTYPE.itemsize
        _olib = lib
    return _olib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _flatten_sets(sets):
    offs = np.zeros(len(sets) + 1, dtype=np.int32)
    for k, c in enumerate(sets):
        offs[k + 1] = offs[k] + len(c)
    feats = np.array([int(f) for c in sets for f in c] or [0], dtype=np.int32)
    return feats, offs


class OracleLearner:
    """The oracle counterpart of the GPU learner: same inputs, same outputs."""

    def __init__(self, ds, cfg: LearnerConfig):
        self.lib = load()
        self.ds = ds
        self.cfg = cfg
        self.feats = ds.feature_array()
        self.bins = np.ascontiguousarray(ds.bins)
        self.rec = cfg.record()
        self.h = self.lib.orc_learner_create(self.feats.ctypes.data, ds.num_features, self.bins.ctypes.data,
                                             ds.num_data, self.rec.ctypes.data)
        self.num_leaves = int(cfg.num_leaves)

    def __del__(self):
        try:
            self.lib.orc_learner_destroy(self.h)
        except Exception:
            pass

    def train(self, g, h, rows=None):
        g = np.ascontiguousarray(g, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        rows = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        splits = np.zeros(max(self.num_leaves - 1, 1), dtype=SPLIT_DTYPE)
        leaf_values = np.zeros(self.num_leaves, dtype=np.float64)
        nl = self.lib.orc_learner_train(self.h, g.ctypes.data, h.ctypes.data, _ptr(rows),
                                        0 if rows is None else len(rows), splits.ctypes.data,
                                        leaf_values.ctypes.data)
        root = self.lib.orc_learner_root_output(self.h)
        return splits[:nl - 1].copy(), leaf_values[:nl].copy(), root

    def set_threads(self, threads):
        """Worker threads of the per-feature tasks and the block partition (the rayon pool); the
        config's num_threads keeps seeding the stochastic-rounding noise blocks."""
        self.lib.orc_learner_set_threads(self.h, int(threads))

    def add_score(self, leaf_values, score):
        """serial.rs:1974-1990 — score[row] += leaf_values[leaf of row] over the last tree's
        partition; ``score`` (float64, C-contiguous) is updated in place."""
        lv = np.ascontiguousarray(leaf_values, dtype=np.float64)
        assert score.dtype == np.float64 and score.flags.c_contiguous and len(score) == self.ds.num_data
        self.lib.orc_learner_add_score(self.h, lv.ctypes.data, score.ctypes.data)

    def leaf_histogram(self, leaf):
        """The leaf's histogram pool slot after the last tree: ([total group bins, 2] (gradient,
        hessian) float64 or (quantized) int64, the [num_features] mask of the features its last
        search covered — the slot's other entries are left from earlier use); None when the leaf
        has no slot."""
        total = sum(fi.group_bins for fi in self.ds.features)
        out = np.zeros((total, 2), dtype=np.int64 if self.cfg.use_quantized_grad else np.float64)
        used = np.zeros(self.ds.num_features, np.uint8)
        slot = self.lib.orc_learner_leaf_histogram(self.h, int(leaf), out.ctypes.data, used.ctypes.data)
        return None if slot < 0 else (out, used.astype(bool))

    def set_feature_mask(self, mask=None):
        """By-tree column sample of the following trees (None = every feature)."""
        if mask is None:
            self._mask = None
        else:
            self._mask = np.ascontiguousarray(np.asarray(mask, dtype=bool).reshape(-1), dtype=np.uint8)
            assert len(self._mask) == self.ds.num_features
        self.lib.orc_learner_set_feature_mask(self.h, _ptr(self._mask))

    def set_bynode(self, fraction, bytree_active, rng_state):
        self.lib.orc_learner_set_bynode(self.h, float(fraction), int(bool(bytree_active)), int(rng_state))

    def bynode_state(self):
        return int(self.lib.orc_learner_bynode_state(self.h))

    def set_interaction_constraints(self, sets):
        feats, offs = _flatten_sets(sets)
        self.lib.orc_learner_set_interaction_constraints(self.h, feats.ctypes.data, offs.ctypes.data, len(sets))

    def row_leaf(self):
        out = np.zeros(self.ds.num_data, dtype=np.int32)
        self.lib.orc_learner_row_leaf(self.h, out.ctypes.data)
        return out

    def partition(self):
        idx = np.zeros(self.ds.num_data, dtype=np.int32)
        b = np.zeros(self.num_leaves, dtype=np.int64)
        c = np.zeros(self.num_leaves, dtype=np.int64)
        self.lib.orc_learner_partition(self.h, idx.ctypes.data, b.ctypes.data, c.ctypes.data)
        return idx, b, c

    def packed(self):
        out = np.zeros(self.ds.num_data, dtype=np.int16)
        sc = np.zeros(2, dtype=np.float64)
        self.lib.orc_learner_packed(self.h, out.ctypes.data, sc.ctypes.data)
        return out, sc


# ------------------------------------------------------------------------------------------
# objectives (host, f64 score -> f32 gradients), written in the reference's operation order
# ------------------------------------------------------------------------------------------
def bin_dense(X, max_bin=255, min_data_in_bin=3, min_data_in_leaf=20, bin_construct_sample_cnt=200000,
              data_random_seed=1, threads=8):
    """The oracle's own binned dataset of a dense float32 matrix (oracle/binning.cpp: the LCG row
    sample of io/sample.rs, BinMapper::find_bin of io/bin.rs, the stored bins of
    io/dataset.rs:633-685), numerical features, trivial columns dropped (io/dataset.rs:389-393).
    Returns a ``BinnedDataset`` built without the product library."""
    from lgbm_gb300.dataset import BinnedDataset, FeatureInfo
    lib = load()
    X = np.ascontiguousarray(X, dtype=np.float32)
    n, ncol = X.shape
    cap = 1024
    meta = np.zeros((ncol, 4), np.int32)
    nbin = np.zeros(ncol, np.int32)
    bounds = np.zeros((ncol, cap), np.float64)
    bins = np.zeros((ncol, n), np.uint8)
    rc = lib.orc_bin_dense_f32(X.ctypes.data, n, ncol, int(max_bin), int(min_data_in_bin), int(min_data_in_leaf),
                               int(bin_construct_sample_cnt), int(data_random_seed), int(threads), cap,
                               meta.ctypes.data, nbin.ctypes.data, bounds.ctypes.data, bins.ctypes.data)
    if rc != 0:
        raise RuntimeError("orc_bin_dense_f32: bin mapper capacity exceeded")
    feats, keep = [], []
    for c in range(ncol):
        if meta[c, 1]:
            continue
        fi = FeatureInfo()
        fi.real = c
        fi.num_bin = int(nbin[c])
        fi.missing_type = int(meta[c, 0])
        fi.default_bin = int(meta[c, 2])
        fi.most_freq_bin = int(meta[c, 3])
        fi.upper_bounds = bounds[c, :nbin[c]].copy()
        fi.penalty = 1.0
        feats.append(fi)
        keep.append(c)
    return BinnedDataset(bins[keep] if len(keep) < ncol else bins, feats, ncol)


def _madd(a, b, c, fused):
    """utils/common.rs:207-216: a * b + c, rounded once when fused (exact rational arithmetic, one
    correctly rounded conversion), twice otherwise."""
    if fused:
        return float(Fraction(a) * Fraction(b) + Fraction(c))
    return a * b + c


class L2Objective:
    """objective/regression.rs:240-248, :321-330 (weighted) and :127-142."""
    num_class = 1

    def __init__(self, label, weights=None, fused=True):
        self.label = np.asarray(label, dtype=np.float32)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        self.fused = fused
        self.constant_hessian = self.w is None

    def gradients(self, score):
        g = (score - self.label.astype(np.float64)).astype(np.float32)
        if self.w is None:
            h = np.ones_like(g)
        else:
            g = (g * self.w).astype(np.float32)  # f32 product
            h = self.w.copy()
        return g[None, :], h[None, :]

    def boost_from_score(self, k):
        if self.w is None:
            suml = 0.0
            for v in self.label.astype(np.float64):
                suml += v
            return suml / len(self.label)
        suml = sumw = 0.0
        for lab, wt in zip(self.label.astype(np.float64), self.w.astype(np.float64)):
            suml = _madd(float(lab), float(wt), suml, self.fused)
            sumw += float(wt)
        return suml / sumw


class PointwiseRegression:
    """The gradient-only regression objectives of objective/regression.rs:240-318 (unweighted)
    and :349-407 (weighted): huber, fair, poisson, gamma and tweedie, with their initial scores
    (:176-184: the label mean, weighted by madd, and its log for poisson, gamma and tweedie). The
    leaf-renewing forms (l1, quantile, mape) are not restated."""
    num_class = 1

    def __init__(self, kind, label, params, weights=None, fused=True):
        self.kind = kind
        self.label = np.asarray(label, dtype=np.float32)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        self.fused = fused
        self.alpha = float(params.get("alpha", 0.9))
        self.fair_c = float(params.get("fair_c", 1.0))
        self.max_delta_step = float(params.get("poisson_max_delta_step", 0.7))
        self.rho = float(params.get("tweedie_variance_power", 1.5))
        self.constant_hessian = kind == "huber" and self.w is None

    def gradients(self, score):
        n = len(score)
        g = np.empty(n, np.float32)
        h = np.empty(n, np.float32)
        emds = math.exp(self.max_delta_step)
        rho = self.rho
        for i in range(n):
            sc, lab = float(score[i]), float(self.label[i])
            if self.kind == "huber":
                diff = sc - lab
                sgn = 1.0 if diff > 0 else (-1.0 if diff < 0 else 0.0)
                if self.w is None:
                    g[i] = np.float32(diff if abs(diff) <= self.alpha else sgn * self.alpha)
                    h[i] = 1.0
                else:
                    wi = self.w[i]
                    # the clipped form is an f32 product sign * w, widened, times alpha
                    g[i] = np.float32(diff * float(wi) if abs(diff) <= self.alpha
                                      else float(np.float32(sgn) * wi) * self.alpha)
                    h[i] = wi
                continue
            wi = 1.0 if self.w is None else float(self.w[i])
            if self.kind == "fair":
                x, c = sc - lab, self.fair_c
                gv, hv = c * x / (abs(x) + c), c * c / ((abs(x) + c) * (abs(x) + c))
            elif self.kind == "poisson":
                e = math.exp(sc)
                gv, hv = e - lab, e * emds
            elif self.kind == "gamma":
                e = math.exp(-sc)
                gv, hv = _madd(-lab, e, 1.0, self.fused), lab * e
            else:  # tweedie
                e1 = math.exp((1.0 - rho) * sc)
                e2 = math.exp((2.0 - rho) * sc)
                gv = _madd(-lab, e1, e2, self.fused)
                hv = _madd(-lab * (1.0 - rho), e1, (2.0 - rho) * e2, self.fused)
            if self.w is None:
                g[i], h[i] = np.float32(gv), np.float32(hv)
            else:
                g[i], h[i] = np.float32(gv * wi), np.float32(hv * wi)
        return g[None, :], h[None, :]

    def boost_from_score(self, k):
        mean = L2Objective(self.label, self.w, self.fused).boost_from_score(k)
        if self.kind in ("huber", "fair"):
            return mean
        return math.log(mean) if mean > 0.0 else -math.inf


def _percentile(vals, alpha, f32, fused):
    """regression.rs:413-437 (upstream's PercentileFun): interpolate between the order statistics
    around (n - 1) * (1 - alpha) counted from the largest, v1 - (v1 - v2) * bias as one madd;
    ``f32`` values take their difference in f32."""
    n = len(vals)
    if n <= 1:
        return vals[0]
    float_pos = (n - 1) * (1.0 - alpha)
    pos = int(float_pos) + 1
    if pos < 1:
        return max(vals)
    if pos >= n:
        return min(vals)
    bias = float_pos - (pos - 1)
    desc = sorted(vals, reverse=True)
    v1, v2 = desc[pos - 1], desc[pos]
    diff = float(np.float32(v1) - np.float32(v2)) if f32 else v1 - v2
    out = _madd(-diff, bias, float(v1), fused)
    return float(np.float32(out)) if f32 else out


def _weighted_percentile(vals, weights, alpha, f32, fused):
    """regression.rs:439-478 (upstream's WeightedPercentileFun): a stable ascending sort, the f64
    cumulative weights, the first position above alpha of the total, and a linear interpolation
    when that step carries a weight of at least 1."""
    n = len(vals)
    if n <= 1:
        return vals[0]
    idx = sorted(range(n), key=lambda i: vals[i])
    cdf = []
    acc = 0.0
    for j, i in enumerate(idx):
        acc = float(weights[i]) if j == 0 else acc + float(weights[i])
        cdf.append(acc)
    threshold = cdf[n - 1] * alpha
    pos = min(int(np.searchsorted(np.asarray(cdf), threshold, side="right")), n - 1)
    if pos == 0 or pos == n - 1:
        return vals[idx[pos]]
    v1, v2 = vals[idx[pos - 1]], vals[idx[pos]]
    if cdf[pos] - cdf[pos - 1] >= 1.0:
        t = (threshold - cdf[pos - 1]) / (cdf[pos] - cdf[pos - 1])
        diff = float(np.float32(v2) - np.float32(v1)) if f32 else v2 - v1
        out = _madd(t, diff, float(v1), fused)
        return float(np.float32(out)) if f32 else out
    return v1


class RenewingRegression:
    """The leaf-renewing regression objectives of objective/regression.rs: l1, quantile and mape
    (gradients :215-255 and :331-384; initial scores :185-195 from the label's (weighted)
    percentile; after each tree, every leaf's output becomes the (weighted) percentile of its
    rows' residuals label - score, :209-238, called per leaf by boosting/train.rs:1198-1211 before
    shrinkage, on the leaf's rows in partition order)."""
    num_class = 1

    def __init__(self, kind, label, params, weights=None, fused=True):
        self.kind = kind
        self.label = np.asarray(label, dtype=np.float32)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        self.fused = fused
        self.alpha_f32 = np.float32(params.get("alpha", 0.9))
        self.alpha = 0.5 if kind in ("l1", "mape") else float(self.alpha_f32)
        self.constant_hessian = kind == "mape" or self.w is None
        if kind == "mape":
            lw = np.float32(1.0) / np.maximum(np.abs(self.label), np.float32(1.0))
            self.label_weight = (lw if self.w is None else lw * self.w).astype(np.float32)

    def gradients(self, score):
        n = len(score)
        g = np.empty(n, np.float32)
        h = np.ones(n, np.float32) if self.w is None else self.w.copy()
        for i in range(n):
            diff = float(score[i]) - float(self.label[i])
            sgn = np.float32(1.0 if diff > 0 else (-1.0 if diff < 0 else 0.0))
            if self.kind == "l1":
                g[i] = sgn if self.w is None else sgn * self.w[i]
            elif self.kind == "quantile":
                v = np.float32(1.0) - self.alpha_f32 if np.float32(diff) >= 0 else -self.alpha_f32
                g[i] = v if self.w is None else v * self.w[i]
            else:  # mape
                g[i] = sgn * self.label_weight[i]
        return g[None, :], h[None, :]

    def _pct(self, vals, weights, f32):
        if weights is None:
            return _percentile(vals, self.alpha, f32, self.fused)
        return _weighted_percentile(vals, weights, self.alpha, f32, self.fused)

    def boost_from_score(self, k):
        vals = [float(v) for v in self.label]
        weights = self.label_weight if self.kind == "mape" else self.w
        return self._pct(vals, weights, True)

    def renew_tree_output(self, score, rows):
        vals = [float(self.label[r]) - float(score[r]) for r in rows]
        weights = self.label_weight if self.kind == "mape" else self.w
        return self._pct(vals, None if weights is None else weights[rows], False)


class CrossEntropyObjective:
    """objective/xentropy.rs: cross_entropy (:62-91) and cross_entropy_lambda (:127-155), labels in
    [0, 1], optional weights; initial scores from the (madd-weighted) label mean (:36-51)."""
    num_class = 1
    constant_hessian = False

    def __init__(self, label, weights=None, fused=True, lam=False):
        self.label = np.asarray(label, dtype=np.float32)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        self.fused = fused
        self.lam = lam

    def gradients(self, score):
        n = len(score)
        g = np.empty(n, np.float32)
        h = np.empty(n, np.float32)
        for i in range(n):
            sc, lab = float(score[i]), float(self.label[i])
            if self.lam:
                if self.w is None:
                    z = 1.0 / (1.0 + math.exp(-sc))
                    g[i], h[i] = np.float32(z - lab), np.float32(z * (1.0 - z))
                    continue
                w = float(self.w[i])
                epf = math.exp(sc)
                z = 1.0 - math.exp(-w * math.log1p(epf))
                g[i] = np.float32((1.0 - lab / z) * w / (1.0 + 1.0 / epf))
                c = 1.0 / (1.0 - z)
                d = 1.0 + epf
                a = w * epf / (d * d)
                d = c - 1.0
                b = (c / (d * d)) * (_madd(w, epf, 1.0, self.fused) - c)
                h[i] = np.float32(a * _madd(lab, b, 1.0, self.fused))
                continue
            if sc > -37.0:
                e = math.exp(-sc)
                gi = _madd(-lab, e, float(np.float32(1.0) - self.label[i]), self.fused) / (1.0 + e)
                hi = e / ((1.0 + e) * (1.0 + e))
            else:
                e = math.exp(sc)
                gi, hi = e - lab, e
            if self.w is None:
                g[i], h[i] = np.float32(gi), np.float32(hi)
            else:
                w = float(self.w[i])
                g[i], h[i] = np.float32(gi * w), np.float32(hi * w)
        return g[None, :], h[None, :]

    def boost_from_score(self, k):
        mean = L2Objective(self.label, self.w, self.fused).boost_from_score(k)
        if self.lam:
            return math.log(math.expm1(mean))
        pavg = max(min(mean, 1.0 - EPS), EPS)
        return math.log(pavg / (1.0 - pavg))


class BinaryObjective:
    """objective/binary.rs:13-115 (sigmoid, is_unbalance / scale_pos_weight, optional weights)."""
    constant_hessian = False
    num_class = 1

    def __init__(self, label, sigmoid=1.0, weights=None, is_unbalance=False, scale_pos_weight=1.0):
        self.is_pos = np.asarray(label, dtype=np.float32) > 0
        self.s = float(sigmoid)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        # per-class label weights (binary.rs:33-41): is_unbalance up-weights the rarer class by the
        # count ratio, then the positive class is scaled by scale_pos_weight
        pos = int(np.sum(self.is_pos))
        neg = len(self.is_pos) - pos
        self.label_weights = [1.0, 1.0]
        if is_unbalance and pos > 0 and neg > 0:
            if pos > neg:
                self.label_weights[0] = float(pos) / float(neg)
            else:
                self.label_weights[1] = float(neg) / float(pos)
        self.label_weights[1] *= float(scale_pos_weight)

    def gradients(self, score):
        n = len(score)
        g = np.empty(n, np.float32)
        h = np.empty(n, np.float32)
        s = self.s
        for i in range(n):
            label = 1.0 if self.is_pos[i] else -1.0
            lw = self.label_weights[1 if self.is_pos[i] else 0]
            response = -label * s / (1.0 + math.exp(label * s * float(score[i])))
            ar = abs(response)
            if self.w is None:
                g[i] = np.float32(response * lw)
                h[i] = np.float32(ar * (s - ar) * lw)
            else:
                w = float(self.w[i])
                g[i] = np.float32(response * lw * w)
                h[i] = np.float32(ar * (s - ar) * lw * w)
        return g[None, :], h[None, :]

    def boost_from_score(self, k):
        suml = 0.0
        if self.w is None:
            for p in self.is_pos:
                suml += 1.0 if p else 0.0
            sumw = float(len(self.is_pos))
        else:
            sumw = 0.0
            for p, w in zip(self.is_pos, self.w):
                suml += float(np.float32(1.0 if p else 0.0) * w)  # an f32 product, widened
                sumw += float(w)
        pavg = max(min(suml / sumw, 1.0 - EPS), EPS)
        return math.log(pavg / (1.0 - pavg)) / self.s


class OvaObjective:
    """objective/multiclass.rs:114-170: one binary objective per class, class k's positives being
    the rows whose label truncates to k."""
    constant_hessian = False

    def __init__(self, label, num_class, sigmoid=1.0, weights=None, is_unbalance=False, scale_pos_weight=1.0):
        self.num_class = num_class
        lab = np.asarray(label, dtype=np.float32).astype(np.int32)
        self.binary = [BinaryObjective((lab == k).astype(np.float32), sigmoid, weights, is_unbalance,
                                       scale_pos_weight) for k in range(num_class)]

    def gradients(self, score):
        gh = [b.gradients(score[k]) for k, b in enumerate(self.binary)]
        return np.concatenate([g for g, _ in gh]), np.concatenate([h for _, h in gh])

    def boost_from_score(self, k):
        return self.binary[k].boost_from_score(0)

    def class_need_train(self, k):
        pos = self.binary[k].is_pos
        return bool(pos.any()) and not bool(pos.all())


class SoftmaxObjective:
    """objective/multiclass.rs:20-110 (optional weights)."""
    constant_hessian = False

    def __init__(self, label, num_class, weights=None):
        self.num_class = num_class
        self.label_int = np.asarray(label, dtype=np.float32).astype(np.int64)
        self.factor = num_class / (num_class - 1.0)
        self.w = None if weights is None else np.asarray(weights, dtype=np.float32)
        probs = [0.0] * num_class
        if self.w is None:
            for v in self.label_int:
                probs[v] += 1.0
            sum_weight = float(len(self.label_int))
        else:
            sum_weight = 0.0
            for v, w in zip(self.label_int, self.w):
                probs[v] += float(w)
                sum_weight += float(w)
        self.init_probs = np.array([pr / sum_weight for pr in probs])

    def gradients(self, score):
        K = self.num_class
        n = score.shape[1]
        g = np.empty((K, n), np.float32)
        h = np.empty((K, n), np.float32)
        for i in range(n):
            rec = [float(score[k, i]) for k in range(K)]
            wmax = rec[0]
            for v in rec[1:]:
                wmax = max(v, wmax)
            wsum = 0.0
            for k in range(K):
                rec[k] = math.exp(rec[k] - wmax)
                wsum += rec[k]
            for k in range(K):
                rec[k] = rec[k] / wsum
            for k in range(K):
                p = rec[k]
                gi = p - 1.0 if self.label_int[i] == k else p
                hi = self.factor * p * (1.0 - p)
                if self.w is not None:
                    w = float(self.w[i])
                    gi, hi = gi * w, hi * w
                g[k, i] = np.float32(gi)
                h[k, i] = np.float32(hi)
        return g, h

    def boost_from_score(self, k):
        return math.log(max(EPS, self.init_probs[k]))

    def class_need_train(self, k):
        p = abs(self.init_probs[k])
        return not (p <= EPS or p >= 1.0 - EPS)


def make_objective(params, y, weights=None, fused=True):
    obj = params.get("objective", "regression")
    if obj in ("regression", "l2", "regression_l2", "mse"):
        if params.get("reg_sqrt", False):
            # regression.rs:50-71: the model is fitted to sign(y) * sqrt(|y|), an f32 label
            y = np.sign(np.asarray(y, np.float32)) * np.sqrt(np.abs(np.asarray(y, np.float32)))
        return L2Objective(y, weights, fused)
    if obj in ("cross_entropy", "xentropy", "cross_entropy_lambda", "xentlambda"):
        return CrossEntropyObjective(y, weights, fused, lam=obj in ("cross_entropy_lambda", "xentlambda"))
    if obj in ("regression_l1", "l1", "mae", "quantile", "mape"):
        return RenewingRegression("l1" if obj in ("regression_l1", "l1", "mae") else obj, y, params, weights, fused)
    if obj in ("huber", "fair", "poisson", "gamma", "tweedie"):
        return PointwiseRegression(obj, y, params, weights, fused)
    if obj == "binary":
        return BinaryObjective(y, params.get("sigmoid", 1.0), weights, bool(params.get("is_unbalance", False)),
                               float(params.get("scale_pos_weight", 1.0)))
    if obj in ("multiclassova", "multiclass_ova", "ova", "ovr"):
        return OvaObjective(y, int(params["num_class"]), params.get("sigmoid", 1.0), weights,
                            bool(params.get("is_unbalance", False)), float(params.get("scale_pos_weight", 1.0)))
    if obj in ("multiclass", "softmax"):
        return SoftmaxObjective(y, int(params["num_class"]), weights)
    raise ValueError("objective %r is outside the learner's scope" % obj)


# ------------------------------------------------------------------------------------------
# row and column sampling (the Trainer's side of the learner's `rows` / feature-mask inputs)
# ------------------------------------------------------------------------------------------
class TreeColumnSampler:
    """ColSampler (treelearner/col_sampler.rs:9-177, no interaction constraints): the by-tree draw
    once when the learner is built and once per tree (serial.rs:678) on the host; the by-node draws
    of a tree (one per searched leaf) by the learner, continuing the same LCG stream. Features are
    the learner's inner features, which follow the real-index order of the used features."""

    def __init__(self, num_features, fraction, seed, fraction_bynode=1.0, interaction_constraints=None):
        self.nf = num_features
        self.rand = LcgRandom(seed)
        self.icons = interaction_constraints or []
        self._set_on = set()
        self.active = fraction < 1.0
        self.bynode = float(fraction_bynode)
        self.cnt = max(min(1, num_features), int(num_features * fraction + 0.5)) if self.active else num_features
        self.mask = np.ones(num_features, dtype=bool)
        self.reset_by_tree()

    def before_tree(self, learner):
        """reset_by_tree on the host, then the learner draws the by-node samples of the tree from the
        same LCG stream; after the tree the host continues from the learner's state."""
        mask = self.reset_by_tree()
        learner.set_feature_mask(mask)
        if self.icons and id(learner) not in self._set_on:
            learner.set_interaction_constraints(self.icons)
            self._set_on.add(id(learner))
        if self.bynode < 1.0:
            learner.set_bynode(self.bynode, self.active, self.rand.x)

    def after_tree(self, learner):
        if self.bynode < 1.0:
            self.rand.x = learner.bynode_state()

    def reset_by_tree(self):
        if self.active:
            self.mask = np.zeros(self.nf, dtype=bool)
            self.mask[np.asarray(self.rand.sample(self.nf, self.cnt), dtype=np.int64)] = True
        return self.mask.copy()


class RowBagging:
    """Bagging (boosting/sample.rs:16-240 without the by-query / GOSS forms): one LCG per 1024-row
    block seeded bagging_seed + block, one draw per row in row order, redrawn every bagging_freq
    iterations; a row is kept when its draw is below bagging_fraction, or, balanced by label
    (sample.rs:95-104,224-236; binary objective with positives only), below pos_bagging_fraction
    for label > 0 and neg_bagging_fraction otherwise. sample(iter) returns the ascending bag or
    None (all rows)."""
    BLOCK = 1024

    def __init__(self, n, fraction, freq, seed, pos_fraction=1.0, neg_fraction=1.0, positive=None):
        self.n = n
        self.fraction = float(fraction)
        self.freq = int(freq)
        self.positive = None if positive is None else np.asarray(positive, dtype=bool)
        self.balanced = ((float(pos_fraction) < 1.0 or float(neg_fraction) < 1.0)
                         and self.positive is not None and bool(self.positive.any()))
        self.threshold = (np.where(self.positive, float(pos_fraction), float(neg_fraction)) if self.balanced
                          else np.full(n, self.fraction))
        self.active = (self.fraction < 1.0 or self.balanced) and self.freq > 0
        self.rands = [LcgRandom((int(seed) + b) & 0xFFFFFFFF) for b in range((n + self.BLOCK - 1) // self.BLOCK)]
        self.bag = None
        self.need = True

    def sample(self, it):
        if not self.active:
            return None
        if self.need or (len(self.bag) < self.n and it % self.freq == 0):
            self.need = False
            self.bag = np.array([i for i in range(self.n)
                                 if float(self.rands[i // self.BLOCK].next_float()) < self.threshold[i]],
                                dtype=np.int32)
        return self.bag if len(self.bag) < self.n else None


class Goss:
    """GOSS row sampling (boosting/sample.rs Goss::draw, one tree per iteration): no sampling for
    the first int(1 / learning_rate) iterations; then the rows whose |g * h| (f32) reaches the
    top_rate-th largest value, plus a draw of the rest (one LCG per 1024-row block) whose
    gradients and hessians are scaled by (n - top_k) / other_k in f32."""
    BLOCK = 1024

    def __init__(self, n, top_rate, other_rate, learning_rate, seed):
        self.n = n
        self.top_rate, self.other_rate = float(top_rate), float(other_rate)
        self.warmup = int(1.0 / float(learning_rate))
        self.rands = [LcgRandom((int(seed) + b) & 0xFFFFFFFF) for b in range((n + self.BLOCK - 1) // self.BLOCK)]

    def sample(self, it, g, h):
        """Returns the rows (or None) and rescales g / h ([1, n] float32) in place."""
        if it < self.warmup:
            return None
        n = self.n
        tmp = np.abs((g[0] * h[0]).astype(np.float32))
        top_k = max(int(n * self.top_rate), 1)
        other_k = int(n * self.other_rate)
        threshold = np.sort(tmp)[::-1][top_k - 1]
        multiply = np.float32(np.float32(n - top_k) / np.float32(other_k))
        bag, big = [], 0
        for i in range(n):
            if tmp[i] >= threshold:
                bag.append(i)
                big += 1
            else:
                rest_need = other_k - (len(bag) - big)
                rest_all = (n - i) - (top_k - big)
                prob = rest_need / float(rest_all)
                if float(self.rands[i // self.BLOCK].next_float()) < prob:
                    bag.append(i)
                    g[0, i] = np.float32(g[0, i] * multiply)
                    h[0, i] = np.float32(h[0, i] * multiply)
        bag = np.array(bag, dtype=np.int32)
        return bag if len(bag) < n else None


def resolved_params(model_text):
    """The resolved config a model file records in its parameters section (`[name: value]`
    lines), e.g. the seeds upstream derives from `seed`."""
    out = {}
    for line in model_text.splitlines():
        if line.startswith("[") and line.endswith("]") and ": " in line:
            k, v = line[1:-1].split(": ", 1)
            out[k] = v
    return out


def parse_interaction_constraints(text):
    """`[0,1,2],[3,4,5]` (the model file's parameter line) -> [[0, 1, 2], [3, 4, 5]]."""
    import re
    return [[int(v) for v in grp.split(",") if v.strip()] for grp in re.findall(r"\[([^\]]*)\]", text or "")]


def samplers_from_params(resolved, ds, label=None):
    """(TreeColumnSampler or None, RowBagging or None) for a resolved config; ``label`` enables
    bagging balanced by label for the binary objective."""
    ff = float(resolved.get("feature_fraction", 1))
    fn = float(resolved.get("feature_fraction_bynode", 1))
    icons = parse_interaction_constraints(resolved.get("interaction_constraints", ""))
    cols = (TreeColumnSampler(ds.num_features, ff, int(resolved.get("feature_fraction_seed", 2)), fn, icons)
            if ff < 1 or fn < 1 or icons else None)
    if resolved.get("data_sample_strategy", "bagging") == "goss":
        return cols, Goss(ds.num_data, float(resolved["top_rate"]), float(resolved["other_rate"]),
                          float(resolved["learning_rate"]), int(resolved.get("bagging_seed", 3)))
    positive = (np.asarray(label, dtype=np.float32) > 0
                if label is not None and resolved.get("objective") == "binary" else None)
    bag = RowBagging(ds.num_data, float(resolved.get("bagging_fraction", 1)), int(resolved.get("bagging_freq", 0)),
                     int(resolved.get("bagging_seed", 3)), float(resolved.get("pos_bagging_fraction", 1)),
                     float(resolved.get("neg_bagging_fraction", 1)), positive)
    return cols, (bag if bag.active else None)


def replay_leaves(tree, ds, rows):
    """Leaf of each of `rows` under `tree`, routed on the stored bins with the training routing
    (serial.rs:2009-2041 add_prediction_for_rows; data_partition.rs:299-410 per split)."""
    lib = load()
    feats = ds.feature_array()
    ni = tree.num_leaves - 1
    luts = np.zeros((max(ni, 1), 256), dtype=np.uint8)
    for node in range(ni):
        f = int(tree.split_feature_inner[node])
        if node in tree.cat_bin_bits:
            bits = np.ascontiguousarray(tree.cat_bin_bits[node], dtype=np.uint32)
            lib.orc_route_table_cat(feats[f:f + 1].ctypes.data, bits.ctypes.data, luts[node].ctypes.data)
        else:
            lib.orc_route_table(feats[f:f + 1].ctypes.data, int(tree.threshold_in_bin[node]),
                                int((int(tree.decision_type[node]) >> 1) & 1), luts[node].ctypes.data)
    rows = np.asarray(rows, dtype=np.int64)
    node = np.zeros(len(rows), dtype=np.int64)
    leaf = np.full(len(rows), -1 if ni > 0 else 0, dtype=np.int64)
    live = np.arange(len(rows)) if ni > 0 else np.zeros(0, np.int64)
    while len(live):
        nd = node[live]
        b = ds.bins[tree.split_feature_inner[nd], rows[live]]
        nxt = np.where(luts[nd, b] != 0, tree.left_child[nd], tree.right_child[nd]).astype(np.int64)
        done = nxt < 0
        leaf[live[done]] = ~nxt[done]
        node[live[~done]] = nxt[~done]
        live = live[~done]
    return leaf


def train_rf(learner, ds, objective, rounds, min_gain_to_split=0.0, col_sampler=None, bagging=None):
    """Random forest boosting (boosting/train.rs:600-608,637-700): the gradients are taken once at
    the initial score; each iteration's trees are grown on a fresh row sample of those same
    gradients, renewed against the initial score, carry the initial score as a bias and are not
    shrunk. Returns the trees."""
    K = getattr(objective, "num_class", 1)
    n = ds.num_data
    init = [0.0] * K
    for k in range(K):
        v = objective.boost_from_score(k)
        init[k] = v if abs(v) > EPS else 0.0
    pred = np.repeat(np.asarray(init, dtype=np.float64)[:, None], n, axis=1)
    g, h = objective.gradients(pred[0] if K == 1 else pred)
    trees = []
    for it in range(rounds):
        rows = bagging.sample(it) if bagging is not None else None
        for k in range(K):
            if col_sampler is not None:
                col_sampler.before_tree(learner)
            recs, leaf_values, root = learner.train(g[k], h[k], rows)
            if col_sampler is not None:
                col_sampler.after_tree(learner)
            t = Tree.from_records(learner.num_leaves, recs, leaf_values, root, ds.features, min_gain_to_split)
            if t.num_leaves > 1:
                if hasattr(objective, "renew_tree_output"):
                    leaf = learner.row_leaf()
                    for lf in range(t.num_leaves):
                        rows_lf = np.nonzero(leaf == lf)[0]
                        if len(rows_lf):
                            t.leaf_value[lf] = _round_to_zero(objective.renew_tree_output(pred[k], rows_lf))
                if abs(init[k]) > EPS:
                    t.add_bias(init[k])
            trees.append(t)
    return trees


def train_gbdt(learner, ds, objective, rounds, learning_rate=0.1, boost_from_average=True,
               min_gain_to_split=0.0, col_sampler=None, bagging=None):
    """train.rs:723-839 with optional bagging or GOSS (rows passed to the learner, out-of-bag rows
    scored by replaying the tree, serial.rs:1995-2000), a column sampler (a mask set before each
    tree) and the objective's leaf renewal before shrinkage (train.rs:780-783); no DART / RF.
    Returns (trees, score)."""
    K = getattr(objective, "num_class", 1)
    n = ds.num_data
    score = np.zeros((K, n), dtype=np.float64)
    trees = []
    for it in range(rounds):
        init = [0.0] * K
        for k in range(K):
            if it == 0 and boost_from_average:
                v = objective.boost_from_score(k)
                if abs(v) > EPS:
                    init[k] = v
                    score[k] += v
        g, h = objective.gradients(score[0] if K == 1 else score)
        if isinstance(bagging, Goss):
            rows = bagging.sample(it, g, h)
        else:
            rows = bagging.sample(it) if bagging is not None else None
        oob = None if rows is None else np.setdiff1d(np.arange(n, dtype=np.int32), rows)
        cont = False
        for k in range(K):
            need = objective.class_need_train(k) if hasattr(objective, "class_need_train") else True
            if not need:
                raise NotImplementedError("constant class trees are outside the learner's scope")
            if col_sampler is not None:
                col_sampler.before_tree(learner)
            recs, leaf_values, root = learner.train(g[k], h[k], rows)
            if col_sampler is not None:
                col_sampler.after_tree(learner)
            t = Tree.from_records(learner.num_leaves, recs, leaf_values, root, ds.features, min_gain_to_split)
            if t.num_leaves > 1:
                cont = True
                leaf = learner.row_leaf()
                if hasattr(objective, "renew_tree_output"):
                    for lf in range(t.num_leaves):
                        rows_lf = np.nonzero(leaf == lf)[0]  # ascending: the stable partition's order
                        if len(rows_lf):
                            t.leaf_value[lf] = _round_to_zero(objective.renew_tree_output(score[k], rows_lf))
                t.apply_shrinkage(learning_rate)
                inbag = leaf >= 0
                score[k][inbag] += t.leaf_value[leaf[inbag]]
                if oob is not None and len(oob):
                    score[k][oob] += t.leaf_value[replay_leaves(t, ds, oob)]
                if abs(init[k]) > EPS:
                    t.add_bias(init[k])
            trees.append(t)
        if not cont:
            trees = trees[:-K]
            break
    return trees, score


# ------------------------------------------------------------------------------------------
# model text
# ------------------------------------------------------------------------------------------
def parse_model_trees(text):
    trees = []
    cur = None
    for line in text.splitlines():
        if line.startswith("Tree="):
            cur = {}
            trees.append(cur)
            continue
        if cur is None or "=" not in line:
            if line.strip() == "end of trees":
                break
            continue
        k, v = line.split("=", 1)
        cur[k] = v
    return trees


def compare_tree(t: Tree, ref: dict, leaf_rtol=1e-12):
    """Returns a list of mismatch descriptions (empty when the tree matches)."""
    bad = []
    nl = int(ref["num_leaves"])
    if t.num_leaves != nl:
        return ["num_leaves %d != %d" % (t.num_leaves, nl)]
    ni = nl - 1

    def ints(key):
        return np.array([int(x) for x in ref[key].split()], dtype=np.int64) if ni or key.startswith("leaf") else \
            np.zeros(0, np.int64)

    def floats(key):
        return np.array([float(x) for x in ref[key].split()], dtype=np.float64)

    if ni > 0:
        for key, mine in (("split_feature", t.split_feature[:ni]), ("decision_type", t.decision_type[:ni]),
                          ("left_child", t.left_child[:ni]), ("right_child", t.right_child[:ni]),
                          ("internal_count", t.internal_count[:ni])):
            if not np.array_equal(ints(key), mine.astype(np.int64)):
                bad.append(key)
        if not np.array_equal(floats("threshold"), t.threshold[:ni]):
            bad.append("threshold")
        if not np.allclose(floats("split_gain"), t.split_gain[:ni].astype(np.float64), rtol=1e-5, atol=1e-12):
            bad.append("split_gain")
        if not np.allclose(floats("internal_value"), t.internal_value[:ni], rtol=1e-5, atol=1e-9):
            bad.append("internal_value")
        if not np.allclose(floats("internal_weight"), t.internal_weight[:ni], rtol=1e-5):
            bad.append("internal_weight")
    if int(ref.get("num_cat", "0")) != t.num_cat:
        bad.append("num_cat")
    elif t.num_cat > 0:
        if [int(x) for x in ref["cat_boundaries"].split()] != t.cat_boundaries:
            bad.append("cat_boundaries")
        if [int(x) for x in ref["cat_threshold"].split()] != t.cat_threshold:
            bad.append("cat_threshold")
    if not np.array_equal(ints("leaf_count"), t.leaf_count[:nl].astype(np.int64)):
        bad.append("leaf_count")
    if not np.allclose(floats("leaf_value"), t.leaf_value[:nl], rtol=leaf_rtol, atol=0):
        bad.append("leaf_value")
    if ni > 0 and not np.allclose(floats("leaf_weight"), t.leaf_weight[:nl], rtol=1e-12):
        bad.append("leaf_weight")
    return bad


# ---------------------------------------------------------------------------------------------
# Error report of a GPU tree against the oracle's f64 learner (the checker, not the thing timed).
# ---------------------------------------------------------------------------------------------
def current_leaves(records, min_data_in_leaf, max_depth=-1):
    """Leaves whose histogram pool slot holds their own final histogram after the tree: every leaf
    searched after the split that made it (serial.rs:779-825 BeforeFindBestSplit let it through),
    except the last split's two children, which no search follows. records: the split records in
    order (SPLIT_DTYPE)."""
    n = len(records)
    if n == 0:
        return [0]
    depth = {0: 0}
    last = {}
    for i, r in enumerate(records):
        bl, nl = int(r["leaf"]), int(r["right_leaf"])
        d = depth.get(bl, 0) + 1
        depth[bl] = depth[nl] = d
        lc, rc = int(r["left_count"]), int(r["right_count"])
        go = not (max_depth > 0 and d >= max_depth) and not (lc < 2 * min_data_in_leaf and rc < 2 * min_data_in_leaf)
        last[bl] = last[nl] = (i, go)
    return sorted(leaf for leaf, (i, go) in last.items() if go and i < n - 1)


def searched_entries(ds, used):
    """Mask over the group bins of a slot: the searched slice (group bins 1 .. num_bin - offset;
    group bin 0 is the elided most-frequent bin, outside every search) of the features in `used`."""
    mask = []
    for fi, u in zip(ds.features, used):
        m = np.zeros(fi.group_bins, bool)
        m[1:] = bool(u)
        mask.append(m)
    return np.concatenate(mask)


def histogram_errors(ds, row_leaf, g, h, leaves, gpu_hist, orc_hist):
    """Error of the device float histograms against the oracle's f64 sums over the searched slice
    of every feature the leaf's last search covered (group bins 1 .. num_bin - offset; group bin 0
    is the elided most-frequent bin, outside every search). gpu_hist: leaf -> [total group bins,
    2]; orc_hist: leaf -> (that, the searched-feature mask). Each entry's
    error is |gpu - oracle| divided by the entry's absolute mass (the sum of |gradient| or of the
    hessians of the rows behind it: serial.rs:1167-1207 FixHistogram gives the most frequent bin
    the leaf total minus the other bins); entries whose mass is below 1e-9 of the feature's mass in
    the leaf are reported only relative to that feature mass. Returns max / mean relative errors
    and the count."""
    gstart = np.cumsum([0] + [fi.group_bins for fi in ds.features])
    rel, rel_leaf = [], []
    ag, hh = np.abs(np.asarray(g, np.float64)), np.asarray(h, np.float64)
    for leaf in leaves:
        rows = np.flatnonzero(row_leaf == leaf)
        a, (b, used) = gpu_hist[leaf], orc_hist[leaf]
        for j, fi in enumerate(ds.features):
            if not used[j]:
                continue
            gb = fi.group_bins
            col = np.asarray(ds.bins[j][rows], dtype=np.int64)
            mass = np.stack([np.bincount(col, weights=ag[rows], minlength=gb),
                             np.bincount(col, weights=hh[rows], minlength=gb)], axis=1)
            if fi.most_freq_bin > 0:  # the fixed entry holds the stored-bin-0 rows
                mass[fi.most_freq_bin + 1] = mass[0]
            sl = slice(gstart[j] + 1, gstart[j] + gb)
            d = np.abs(a[sl] - b[sl])
            m = mass[1:]
            fm = m.sum(axis=0, keepdims=True)
            ok = m > 1e-9 * fm
            rel.append(d[ok] / m[ok])
            rel_leaf.append((d / np.maximum(fm, 1e-300)).ravel())
    rel = np.concatenate(rel) if rel else np.zeros(0)
    rel_leaf = np.concatenate(rel_leaf) if rel_leaf else np.zeros(0)
    return {"leaves": len(leaves), "entries": int(rel_leaf.size),
            "max_rel": float(rel.max()) if rel.size else 0.0, "mean_rel": float(rel.mean()) if rel.size else 0.0,
            "max_rel_to_feature_mass": float(rel_leaf.max()) if rel_leaf.size else 0.0}


def gain_errors(rec_gpu, rec_orc):
    """Split-by-split comparison of two float trees grown from the same gradients: relative gain
    error of every split while the two trees agree, and the near-tie divergences (the first split
    whose leaf, feature or threshold differs, with both gains)."""
    rel, near_ties = [], []
    for i, (a, b) in enumerate(zip(rec_gpu, rec_orc)):
        same = (int(a["leaf"]) == int(b["leaf"]) and int(a["real_feature"]) == int(b["real_feature"])
                and int(a["threshold"]) == int(b["threshold"]) and int(a["default_left"]) == int(b["default_left"]))
        ga, gb = float(a["gain"]), float(b["gain"])
        if not same:
            near_ties.append({"split": i, "gpu": [int(a["leaf"]), int(a["real_feature"]), int(a["threshold"]), ga],
                              "oracle": [int(b["leaf"]), int(b["real_feature"]), int(b["threshold"]), gb],
                              "gain_rel_diff": abs(ga - gb) / max(abs(gb), 1e-300)})
            break
        rel.append(abs(ga - gb) / max(abs(gb), 1e-300))
    rel = np.asarray(rel)
    return {"splits_compared": int(rel.size), "max_rel": float(rel.max()) if rel.size else 0.0,
            "mean_rel": float(rel.mean()) if rel.size else 0.0, "near_ties": near_ties}


def split_match(rec_gpu, rec_orc):
    """Whole-tree comparison of two float trees grown from the same gradients, past near-tie
    divergences: every split node is keyed by its path from the root (the (feature, threshold,
    default_left, side) of each ancestor split), which fixes the node's rows. Nodes whose key and
    split agree in both trees are matched (their gains compared); the rest are divergences, listed
    with both trees' choices. A near tie changes the subtree under the node where it happens (and,
    through the leaf budget, which leaves get split at all), not the splits elsewhere."""
    def nodes(rec):
        path = {0: ()}
        out = {}
        for i, r in enumerate(rec):
            leaf, right = int(r["leaf"]), int(r["right_leaf"])
            key = path[leaf]
            sp = (int(r["real_feature"]), int(r["threshold"]), int(r["default_left"]))
            out[key] = (sp, float(r["gain"]), i)
            path[leaf] = key + (sp + (0,),)
            path[right] = key + (sp + (1,),)
        return out
    a, b = nodes(rec_gpu), nodes(rec_orc)
    rel, diverged = [], []
    for key in sorted(set(a) | set(b), key=lambda k: (len(k), k)):
        x, y = a.get(key), b.get(key)
        if x is not None and y is not None and x[0] == y[0]:
            rel.append(abs(x[1] - y[1]) / max(abs(y[1]), 1e-300))
        else:
            diverged.append({"depth": len(key), "gpu": None if x is None else [*x[0], x[1], x[2]],
                             "oracle": None if y is None else [*y[0], y[1], y[2]]})
    rel = np.asarray(rel)
    return {"matched": int(rel.size), "diverged": len(diverged), "splits": (len(rec_gpu), len(rec_orc)),
            "max_rel": float(rel.max()) if rel.size else 0.0, "mean_rel": float(rel.mean()) if rel.size else 0.0,
            "divergences": diverged[:20]}

"""Routing of held-out rows on stored bins against upstream's predictor (no GPU).

Six upstream models of the reference's tests/fixtures (binary, NaN missing values, zero as
missing, L2, a categorical feature, 3-class multiclass), each with its training rows, test rows
and the leaf upstream's predictor sends every test row to in every tree (pred_leaf.npy, which
crates/lgbm-core/tests/golden_predict.rs checks for the reference). The training rows are binned
by the host bin mappers, the test rows with the same mappers, each tree's value thresholds
become bin thresholds (a numerical threshold is one of its feature's bin upper bounds; a
categorical split's category bitset becomes a bin bitset), and the rows are routed on their
stored bins through the route tables of the learner's partition (data_partition.rs:264-410):
every test row must reach upstream's leaf, NaN and zero-as-missing rows and unseen categories
included; and the raw scores, the leaf values summed in tree order, equal upstream's bit for
bit. This is the routing and the score update that bk_learner_predict_add and the out-of-bag
replay use.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

PREDICT = os.path.join(GOLDEN, "predict")
CASES = sorted(os.listdir(PREDICT))


class _Tree:
    """The fields of one model-text tree that routing needs, in bin terms."""

    def __init__(self, rec, ds):
        inner_of = {fi.real: j for j, fi in enumerate(ds.features)}
        self.num_leaves = int(rec["num_leaves"])
        ni = self.num_leaves - 1
        ints = lambda k: np.array([int(v) for v in rec[k].split()], dtype=np.int64) if ni else np.zeros(0, np.int64)
        self.left_child, self.right_child = ints("left_child"), ints("right_child")
        self.decision_type = ints("decision_type").astype(np.int8)
        real = ints("split_feature")
        thr = [float(v) for v in rec["threshold"].split()] if ni else []
        self.split_feature_inner = np.array([inner_of[int(r)] for r in real], dtype=np.int64)
        self.threshold_in_bin = np.zeros(ni, dtype=np.uint32)
        self.cat_bin_bits = {}
        bounds = [int(v) for v in rec.get("cat_boundaries", "0").split()]
        words = [int(v) for v in rec.get("cat_threshold", "").split()]
        for node in range(ni):
            fi = ds.features[self.split_feature_inner[node]]
            if self.decision_type[node] & 1:
                k = int(thr[node])
                cats = words[bounds[k]:bounds[k + 1]]
                bits = np.zeros(8, np.uint32)
                for b in range(1, fi.num_bin):
                    c = int(fi.bin_to_category[b])
                    if c >= 0 and c // 32 < len(cats) and (cats[c // 32] >> (c % 32)) & 1:
                        bits[b // 32] |= np.uint32(1 << (b % 32))
                self.cat_bin_bits[node] = bits
            else:
                hits = np.flatnonzero(fi.upper_bounds == thr[node])
                assert len(hits) == 1, "threshold %r is not a bin bound" % thr[node]
                self.threshold_in_bin[node] = hits[0]


@pytest.mark.parametrize("case", CASES)
def test_held_out_rows_reach_upstreams_leaves(oracle, bklib, case):
    from lgbm_gb300 import BinnedDataset
    d = os.path.join(PREDICT, case)
    P = json.load(open(os.path.join(d, "params.json")))
    train = np.load(os.path.join(d, "train.npy"))
    test = np.load(os.path.join(d, "test.npy"))
    want = np.load(os.path.join(d, "pred_leaf.npy"))
    ds = BinnedDataset.from_dense(train[:, 1:], zero_as_missing=P["params"].get("zero_as_missing", False),
                                  categorical=P["dataset"].get("categorical_feature", []))
    held = BinnedDataset(ds.bin_like(test[:, 1:]), ds.features, ds.num_total_features)
    trees = oracle.parse_model_trees(open(os.path.join(d, "model.txt")).read())
    assert want.shape == (len(test), len(trees))
    rows = np.arange(len(test))
    raw_want = np.load(os.path.join(d, "pred_raw.npy")).reshape(len(test), -1)
    K = raw_want.shape[1]
    raw = np.zeros((len(test), K))
    for k, rec in enumerate(trees):
        got = oracle.replay_leaves(_Tree(rec, ds), held, rows)
        assert np.array_equal(got, want[:, k]), "tree %d: %d of %d rows differ" % (k, int(np.sum(got != want[:, k])),
                                                                                     len(rows))
        # the score update: every tree's leaf value added in tree order (class k % K)
        leaf_value = np.array([float(v) for v in rec["leaf_value"].split()])
        raw[:, k % K] += leaf_value[got]
    assert np.array_equal(raw, raw_want), "raw scores differ"

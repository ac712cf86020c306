"""Host-side tree assembly from the learner's split records.

The learner returns, per split, the arguments of ``Tree::split_numerical``
(crates/lgbm-core/src/tree.rs:361-403) or ``Tree::split_categorical`` (:405-443); this module
applies them exactly like the reference's ``Tree`` (``split_common`` tree.rs:310-357,
``apply_shrinkage`` :446-463, ``add_bias`` :465-478) so the result can be compared with, or
written as, a LightGBM model tree.
"""
import numpy as np

K_ZERO_THRESHOLD = float(np.float32(1e-35))
K_CATEGORICAL_MASK = 1  # tree.rs decision_type bit 0


def construct_bitset(vals):
    """utils/common.rs:221-231: bit v of word v / 32 for every value; as many words as the largest
    value needs."""
    words = []
    for v in vals:
        i1 = v // 32
        if len(words) < i1 + 1:
            words.extend([0] * (i1 + 1 - len(words)))
        words[i1] |= 1 << (v % 32)
    return words


def bits_to_bins(bits):
    """The set bits of an 8-word bin bitset, ascending."""
    return [b for b in range(256) if (int(bits[b // 32]) >> (b % 32)) & 1]

SPLIT_DTYPE = np.dtype([
    ("leaf", np.int32), ("right_leaf", np.int32), ("inner_feature", np.int32), ("real_feature", np.int32),
    ("threshold", np.uint32), ("default_left", np.int32), ("missing_type", np.int32), ("left_count", np.int32),
    ("right_count", np.int32), ("left_output", np.float64), ("right_output", np.float64),
    ("left_sum_gradient", np.float64), ("left_sum_hessian", np.float64), ("right_sum_gradient", np.float64),
    ("right_sum_hessian", np.float64), ("gain", np.float64), ("left_int_sum", np.int64),
    ("right_int_sum", np.int64), ("categorical", np.int32), ("_pad", np.int32), ("cat_bins", np.uint32, (8,)),
], align=True)


def _round_to_zero(v):
    return 0.0 if -K_ZERO_THRESHOLD <= v <= K_ZERO_THRESHOLD else v


class Tree:
    def __init__(self, max_leaves):
        n_int = max(max_leaves - 1, 0)
        self.num_leaves = 1
        self.left_child = np.zeros(n_int, np.int32)
        self.right_child = np.zeros(n_int, np.int32)
        self.split_feature = np.zeros(n_int, np.int32)
        self.split_feature_inner = np.zeros(n_int, np.int32)
        self.split_gain = np.zeros(n_int, np.float32)
        self.threshold = np.zeros(n_int, np.float64)
        self.threshold_in_bin = np.zeros(n_int, np.uint32)
        self.decision_type = np.zeros(n_int, np.int8)
        self.leaf_value = np.zeros(max_leaves, np.float64)
        self.leaf_weight = np.zeros(max_leaves, np.float64)
        self.leaf_count = np.zeros(max_leaves, np.int32)
        self.leaf_parent = np.full(max_leaves, -1, np.int32)
        self.leaf_depth = np.zeros(max_leaves, np.int32)
        self.internal_value = np.zeros(n_int, np.float64)
        self.internal_weight = np.zeros(n_int, np.float64)
        self.internal_count = np.zeros(n_int, np.int32)
        self.shrinkage = 1.0
        # categorical splits (tree.rs:405-443): per node its category bitset range, and the bins
        # that go left (for replays on stored bins)
        self.num_cat = 0
        self.cat_boundaries = [0]
        self.cat_threshold = []
        self.cat_bin_bits = {}

    @classmethod
    def from_records(cls, max_leaves, records, leaf_values, root_output, features, min_gain_to_split=0.0):
        """Rebuild the tree from split records; ``leaf_values`` are the learner's final outputs and
        ``root_output`` the root leaf's output before the first split (serial.rs:580-586)."""
        t = cls(max_leaves)
        t.leaf_value[0] = _round_to_zero(float(root_output))
        for r in records:
            leaf, nl = int(r["leaf"]), t.num_leaves
            node = nl - 1
            parent = t.leaf_parent[leaf]
            if parent >= 0:
                if t.left_child[parent] == ~leaf:
                    t.left_child[parent] = node
                else:
                    t.right_child[parent] = node
            fi = features[int(r["inner_feature"])]
            t.split_feature_inner[node] = r["inner_feature"]
            t.split_feature[node] = r["real_feature"]
            t.split_gain[node] = np.float32(float(r["gain"]) + min_gain_to_split)
            t.left_child[node] = ~leaf
            t.right_child[node] = ~nl
            t.leaf_parent[leaf] = node
            t.leaf_parent[nl] = node
            t.internal_weight[node] = float(r["left_sum_hessian"]) + float(r["right_sum_hessian"])
            t.internal_value[node] = t.leaf_value[leaf]
            t.internal_count[node] = int(r["left_count"]) + int(r["right_count"])
            lo, ro = float(r["left_output"]), float(r["right_output"])
            t.leaf_value[leaf] = 0.0 if np.isnan(lo) else lo
            t.leaf_weight[leaf] = r["left_sum_hessian"]
            t.leaf_count[leaf] = r["left_count"]
            t.leaf_value[nl] = 0.0 if np.isnan(ro) else ro
            t.leaf_weight[nl] = r["right_sum_hessian"]
            t.leaf_count[nl] = r["right_count"]
            t.leaf_depth[nl] = t.leaf_depth[leaf] + 1
            t.leaf_depth[leaf] += 1
            if int(r["categorical"]):
                # the tree keeps the categories of the left bins; the partition used the bins
                bins = bits_to_bins(r["cat_bins"])
                bitset = construct_bitset([int(fi.bin_to_category[b]) for b in bins])
                t.decision_type[node] = K_CATEGORICAL_MASK | (int(r["missing_type"]) << 2)
                t.threshold_in_bin[node] = t.num_cat
                t.threshold[node] = float(t.num_cat)
                t.num_cat += 1
                t.cat_boundaries.append(t.cat_boundaries[-1] + len(bitset))
                t.cat_threshold.extend(bitset)
                t.cat_bin_bits[node] = np.asarray(r["cat_bins"], dtype=np.uint32).copy()
            else:
                dt = 2 if r["default_left"] else 0
                dt = (dt & 3) | (int(r["missing_type"]) << 2)
                t.decision_type[node] = dt
                t.threshold_in_bin[node] = r["threshold"]
                t.threshold[node] = fi.bin_to_value(int(r["threshold"]))
            t.num_leaves += 1
        # the learner's final leaf outputs (equal to the split outputs unless renewed)
        for i in range(t.num_leaves):
            t.leaf_value[i] = float(leaf_values[i])
        return t

    def apply_shrinkage(self, rate):
        n = self.num_leaves
        for i in range(max(n - 1, 0)):
            self.leaf_value[i] = _round_to_zero(self.leaf_value[i] * rate)
            self.internal_value[i] = _round_to_zero(self.internal_value[i] * rate)
        self.leaf_value[n - 1] = _round_to_zero(self.leaf_value[n - 1] * rate)
        self.shrinkage *= rate

    def add_bias(self, val):
        n = self.num_leaves
        for i in range(max(n - 1, 0)):
            self.leaf_value[i] = _round_to_zero(self.leaf_value[i] + val)
            self.internal_value[i] = _round_to_zero(self.internal_value[i] + val)
        self.leaf_value[n - 1] = _round_to_zero(self.leaf_value[n - 1] + val)
        self.shrinkage = 1.0

"""``GpuTreeLearner`` — the host-side mirror of bankai-lightgbm's ``SerialTreeLearner``
(crates/lgbm-core/src/treelearner/serial.rs:183-2044) over the C ABI of ``lib/libbkgpu.so``.

Same constructor inputs (a binned dataset, the learner config, ``is_constant_hessian``), same
``train(gradients, hessians, rows) -> tree`` contract, same score update. Training runs on the
GPU; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _lib
from .config import LearnerConfig
from .tree import SPLIT_DTYPE, Tree


class GpuTreeLearner:
    def __init__(self, ds, cfg: LearnerConfig, num_jobs: int = 1, loop_mode: int = 1):
        self.lib = _lib.load()
        self.ds = ds
        self.cfg = cfg
        self.num_jobs = int(num_jobs)
        self.num_leaves = int(cfg.num_leaves)
        self._feats = ds.feature_array()
        self._rec = cfg.record()
        h = ctypes.c_void_p()
        if ds.on_device:
            # stored bins already in device memory (BinnedDataset.from_dense_device)
            _lib.check(self.lib.bk_learner_create_device_bins(self._feats.ctypes.data, ds.num_features,
                                                              ds.bins.data_ptr(), ds.num_data, self._rec.ctypes.data,
                                                              self.num_jobs, ctypes.byref(h)),
                       "bk_learner_create_device_bins")
        else:
            self._bins = np.ascontiguousarray(ds.bins, dtype=np.uint8)
            _lib.check(self.lib.bk_learner_create(self._feats.ctypes.data, ds.num_features, self._bins.ctypes.data,
                                                  ds.num_data, self._rec.ctypes.data, self.num_jobs, ctypes.byref(h)),
                       "bk_learner_create")
        self.h = h
        self.set_loop_mode(loop_mode)

    def close(self):
        if getattr(self, "h", None):
            self.lib.bk_learner_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_loop_mode(self, mode: int):
        _lib.check(self.lib.bk_learner_set_loop_mode(self.h, int(mode)), "bk_learner_set_loop_mode")

    def set_launch_overlap(self, on: bool):
        """Programmatic dependent launch of the grow-loop kernels (default on)."""
        _lib.check(self.lib.bk_learner_set_launch_overlap(self.h, int(bool(on))), "bk_learner_set_launch_overlap")

    def set_feature_mask(self, mask=None):
        """The by-tree column sample of the following trees (ColSampler::reset_by_tree,
        treelearner/col_sampler.rs:87-103): mask [num_jobs, num_features] (or [num_features] for
        one job) of inner features the trees may split on; None = every feature."""
        if mask is None:
            _lib.check(self.lib.bk_learner_set_feature_mask(self.h, None), "bk_learner_set_feature_mask")
            return
        m = np.ascontiguousarray(np.asarray(mask, dtype=bool).reshape(self.num_jobs, self.ds.num_features),
                                 dtype=np.uint8)
        _lib.check(self.lib.bk_learner_set_feature_mask(self.h, m.ctypes.data), "bk_learner_set_feature_mask")

    def set_bynode(self, fraction, bytree_active, rng_state):
        """The by-node column sample of the following trees (ColSampler::get_by_node,
        treelearner/col_sampler.rs:109-177) drawn on the device, continuing the sampler's LCG
        state ``rng_state`` (after the host's by-tree draw)."""
        _lib.check(self.lib.bk_learner_set_bynode(self.h, float(fraction), int(bool(bytree_active)),
                                                  int(rng_state) & 0xFFFFFFFF), "bk_learner_set_bynode")

    def set_interaction_constraints(self, sets):
        """Interaction constraints of the following trees: a list of sets of real feature indices
        (treelearner/col_sampler.rs:148-177); [] removes them."""
        offs = np.zeros(len(sets) + 1, dtype=np.int32)
        for k, c in enumerate(sets):
            offs[k + 1] = offs[k] + len(c)
        feats = np.array([int(f) for c in sets for f in c] or [0], dtype=np.int32)
        _lib.check(self.lib.bk_learner_set_interaction_constraints(self.h, feats.ctypes.data, offs.ctypes.data,
                                                                   len(sets)),
                   "bk_learner_set_interaction_constraints")

    def bynode_state(self):
        out = ctypes.c_uint32()
        _lib.check(self.lib.bk_learner_bynode_state(self.h, ctypes.byref(out)), "bk_learner_bynode_state")
        return int(out.value)

    def autotune(self, gradients, hessians, on_device=False, trials=2):
        """Picks the grow-loop launch shape by timing whole trees grown from these gradients
        (bk_learner_autotune; cached per dataset shape class). Returns the chosen shape
        (rows per histogram CTA, histogram CTAs per feature tile, partition CTAs, rows per histogram
        CTA up to which it adds to the pool with global atomics, histogram CTAs per cluster)."""
        K = self.num_jobs
        if on_device:
            gp, hp = int(gradients), int(hessians)
        else:
            g = np.ascontiguousarray(gradients, dtype=np.float32).reshape(K, -1)
            hh = np.ascontiguousarray(hessians, dtype=np.float32).reshape(K, -1)
            assert g.shape[1] == self.ds.num_data and hh.shape == g.shape
            gp, hp = g.ctypes.data, hh.ctypes.data
        out = np.zeros(5, np.int32)
        _lib.check(self.lib.bk_learner_autotune(self.h, gp, hp, int(bool(on_device)), int(trials), out.ctypes.data),
                   "bk_learner_autotune")
        return tuple(int(x) for x in out)

    def launch_shape(self):
        out = np.zeros(5, np.int32)
        _lib.check(self.lib.bk_learner_launch_shape(self.h, out.ctypes.data), "bk_learner_launch_shape")
        return tuple(int(x) for x in out)

    def set_launch_shape(self, shape):
        arr = np.ascontiguousarray(tuple(shape) + (0,) * (5 - len(shape)), dtype=np.int32)
        assert arr.shape == (5,)
        _lib.check(self.lib.bk_learner_set_launch_shape(self.h, arr.ctypes.data), "bk_learner_set_launch_shape")

    def set_timing(self, on: bool):
        _lib.check(self.lib.bk_learner_set_timing(self.h, int(bool(on))), "bk_learner_set_timing")

    def last_timing(self):
        t = (ctypes.c_double * 3)()
        _lib.check(self.lib.bk_learner_last_timing(self.h, ctypes.byref(t, 0), ctypes.byref(t, 8),
                                                   ctypes.byref(t, 16)), "bk_learner_last_timing")
        ph = (ctypes.c_double * 2)()
        _lib.check(self.lib.bk_learner_last_phase_timing(self.h, ctypes.byref(ph, 0), ctypes.byref(ph, 8)),
                   "bk_learner_last_phase_timing")
        return {"total_ms": t[0], "hist_ms": t[1], "hist_bytes": t[2], "search_ms": ph[0], "partition_ms": ph[1]}

    def last_step_timing(self):
        """With timing on: [num_leaves - 1, 3] ms of (histogram, search, partition) per grow-loop
        step of the last train call (-1 where a step did not run)."""
        out = np.zeros((self.num_leaves - 1, 3), dtype=np.float32)
        _lib.check(self.lib.bk_learner_last_step_timing(self.h, out.ctypes.data), "bk_learner_last_step_timing")
        return out

    def stream(self):
        s = ctypes.c_void_p()
        _lib.check(self.lib.bk_learner_stream(self.h, ctypes.byref(s)), "bk_learner_stream")
        return s.value

    def objective_gradients(self, kind, score_ptr, label_ptr, sigmoid=1.0):
        _lib.check(self.lib.bk_learner_objective_gradients(self.h, int(kind), int(score_ptr), int(label_ptr),
                                                           float(sigmoid)), "bk_learner_objective_gradients")

    def histogram_cache_capacity(self):
        """Histogram slots the learner keeps (a full pool: num_leaves)."""
        out = ctypes.c_int64()
        _lib.check(self.lib.bk_learner_histogram_cache_capacity(self.h, ctypes.byref(out)),
                   "bk_learner_histogram_cache_capacity")
        return out.value

    def search_threads(self):
        """Threads per split-search CTA of the next train call (64 or 256)."""
        out = ctypes.c_int32()
        _lib.check(self.lib.bk_learner_search_threads(self.h, ctypes.byref(out)), "bk_learner_search_threads")
        return out.value

    def reset_histogram_pool_config(self):
        """The budget-only reset of SerialTreeLearner::reset_histogram_pool_config: nothing changes."""
        _lib.check(self.lib.bk_learner_reset_histogram_pool_config(self.h), "bk_learner_reset_histogram_pool_config")

    def set_objective_weights(self, weights_ptr=0, neg_label_weight=1.0, pos_label_weight=1.0):
        """Row weights (a device f32 [num_data] pointer, 0 for none) and the binary label weights
        used by objective_gradients from now on (bk_learner_set_objective_weights)."""
        _lib.check(self.lib.bk_learner_set_objective_weights(self.h, int(weights_ptr) or None, float(neg_label_weight),
                                                             float(pos_label_weight)),
                   "bk_learner_set_objective_weights")

    def objective_loss(self, kind, score_ptr, label_ptr):
        out = ctypes.c_double()
        _lib.check(self.lib.bk_learner_objective_loss(self.h, int(kind), int(score_ptr), int(label_ptr),
                                                      ctypes.byref(out)), "bk_learner_objective_loss")
        return out.value

    def predict_add(self, tree, bins_ptr, num_rows, score_ptr):
        """Adds `tree`'s output to a device score for device-resident binned rows
        ([num_features][num_rows] uint8 stored bins made with this dataset's bin mappers)."""
        import numpy as np
        ni = max(tree.num_leaves - 1, 0)
        lc = np.ascontiguousarray(tree.left_child[:ni], np.int32)
        rc = np.ascontiguousarray(tree.right_child[:ni], np.int32)
        sf = np.ascontiguousarray(tree.split_feature_inner[:ni], np.int32)
        th = np.ascontiguousarray(tree.threshold_in_bin[:ni], np.uint32)
        dt = np.ascontiguousarray(tree.decision_type[:ni], np.int8)
        lv = np.ascontiguousarray(tree.leaf_value[:tree.num_leaves], np.float64)
        # categorical nodes: the left-bin bitsets (a dict node -> 8 words, or a [ni, 8] array)
        cb = np.zeros((max(ni, 1), 8), np.uint32)
        bits = getattr(tree, "cat_bin_bits", None)
        if bits is not None:
            for node in (bits.keys() if isinstance(bits, dict) else range(ni)):
                cb[node] = np.asarray(bits[node], np.uint32)
        _lib.check(self.lib.bk_learner_predict_add(self.h, tree.num_leaves, lc.ctypes.data, rc.ctypes.data,
                                                   sf.ctypes.data, th.ctypes.data, dt.ctypes.data,
                                                   cb.ctypes.data if bits is not None else None,
                                                   lv.ctypes.data, int(bins_ptr), int(num_rows), int(score_ptr)),
                   "bk_learner_predict_add")

    def gradient_buffers(self):
        g = ctypes.c_void_p()
        h = ctypes.c_void_p()
        _lib.check(self.lib.bk_learner_gradient_buffers(self.h, ctypes.byref(g), ctypes.byref(h)),
                   "bk_learner_gradient_buffers")
        return g.value, h.value

    def train_raw(self, gradients, hessians, rows=None, on_device=False):
        """Trains num_jobs trees. gradients/hessians: [num_jobs, num_data] float32 (numpy), or device
        pointers (int) with on_device=True. Returns (splits, leaf_values, root_outputs, num_leaves)."""
        K, Lv = self.num_jobs, self.num_leaves
        if on_device:
            gp, hp = int(gradients), int(hessians)
        else:
            g = np.ascontiguousarray(gradients, dtype=np.float32).reshape(K, -1)
            hh = np.ascontiguousarray(hessians, dtype=np.float32).reshape(K, -1)
            assert g.shape[1] == self.ds.num_data and hh.shape == g.shape
            gp, hp = g.ctypes.data, hh.ctypes.data
        rows_arr = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        splits = np.zeros((K, max(Lv - 1, 1)), dtype=SPLIT_DTYPE)
        leaf_values = np.zeros((K, Lv), dtype=np.float64)
        roots = np.zeros(K, dtype=np.float64)
        nls = np.zeros(K, dtype=np.int32)
        _lib.check(self.lib.bk_learner_train(self.h, gp, hp, int(bool(on_device)),
                                             None if rows_arr is None else rows_arr.ctypes.data,
                                             0 if rows_arr is None else len(rows_arr), splits.ctypes.data,
                                             leaf_values.ctypes.data, roots.ctypes.data, nls.ctypes.data),
                   "bk_learner_train")
        return splits, leaf_values, roots, nls

    def train(self, gradients, hessians, rows=None):
        """SerialTreeLearner::train for a single job: (splits, leaf_values, root_output)."""
        assert self.num_jobs == 1
        splits, lv, roots, nls = self.train_raw(np.asarray(gradients)[None, :], np.asarray(hessians)[None, :], rows)
        nl = int(nls[0])
        return splits[0, :nl - 1].copy(), lv[0, :nl].copy(), float(roots[0])

    def trees(self, splits, leaf_values, roots, nls):
        return [Tree.from_records(self.num_leaves, splits[j, :nls[j] - 1], leaf_values[j, :nls[j]], roots[j],
                                  self.ds.features, self.cfg.min_gain_to_split) for j in range(self.num_jobs)]

    def row_leaf(self):
        out = np.zeros((self.num_jobs, self.ds.num_data), dtype=np.int32)
        _lib.check(self.lib.bk_learner_row_leaf(self.h, out.ctypes.data), "bk_learner_row_leaf")
        return out[0] if self.num_jobs == 1 else out

    def leaf_histogram(self, leaf, job=0):
        """The histogram pool slot of `leaf` after the last tree (bk_learner_leaf_histogram):
        [total group bins, 2] (gradient, hessian) sums, float64 or (quantized) int64; None when
        the leaf has no slot."""
        total = sum(fi.group_bins for fi in self.ds.features)
        out = np.zeros((total, 2), dtype=np.int64 if self.cfg.use_quantized_grad else np.float64)
        slot = ctypes.c_int32(-2)  # the library writes -1 only for a leaf without a slot
        rc = self.lib.bk_learner_leaf_histogram(self.h, int(job), int(leaf), out.ctypes.data, ctypes.byref(slot))
        if rc != 0:
            if slot.value == -1:
                return None
            _lib.check(rc, "bk_learner_leaf_histogram")
        return out

    def add_prediction_to_score(self, leaf_values, score, on_device=False):
        lv = np.ascontiguousarray(leaf_values, dtype=np.float64).reshape(self.num_jobs, self.num_leaves)
        if on_device:
            _lib.check(self.lib.bk_learner_add_prediction_to_score(self.h, lv.ctypes.data, int(score), 1),
                       "bk_learner_add_prediction_to_score")
        else:
            assert score.dtype == np.float64 and score.flags.c_contiguous
            _lib.check(self.lib.bk_learner_add_prediction_to_score(self.h, lv.ctypes.data, score.ctypes.data, 0),
                       "bk_learner_add_prediction_to_score")


def train_batch(learners, gradients, hessians, on_device=False, shrinkage=None, scores=None):
    """One tree per learner for many independent learners at once (``bk_learners_train_batch``):
    every learner's grow loop is queued on its own stream before any is waited for.

    gradients / hessians: per learner, a [num_jobs, num_data] float32 array, or a device pointer
    (int) with on_device=True. scores: None, or per learner a device pointer to its
    [num_jobs, num_data] f64 score, which then receives the new trees' leaf outputs times
    ``shrinkage``. Returns per learner (splits, leaf_values, root_outputs, num_leaves) as
    ``GpuTreeLearner.train_raw`` does."""
    count = len(learners)
    assert count > 0 and len(gradients) == count and len(hessians) == count
    lib = learners[0].lib
    keep = []
    gp = (ctypes.c_void_p * count)()
    hp = (ctypes.c_void_p * count)()
    for i, L in enumerate(learners):
        if on_device:
            gp[i], hp[i] = int(gradients[i]), int(hessians[i])
        else:
            g = np.ascontiguousarray(gradients[i], dtype=np.float32).reshape(L.num_jobs, -1)
            hh = np.ascontiguousarray(hessians[i], dtype=np.float32).reshape(L.num_jobs, -1)
            assert g.shape[1] == L.ds.num_data and hh.shape == g.shape
            keep += [g, hh]
            gp[i], hp[i] = g.ctypes.data, hh.ctypes.data
    outs = []
    sp = (ctypes.c_void_p * count)()
    lp = (ctypes.c_void_p * count)()
    rp = (ctypes.c_void_p * count)()
    np_ = (ctypes.c_void_p * count)()
    for i, L in enumerate(learners):
        K, Lv = L.num_jobs, L.num_leaves
        o = (np.zeros((K, max(Lv - 1, 1)), dtype=SPLIT_DTYPE), np.zeros((K, Lv), dtype=np.float64),
             np.zeros(K, dtype=np.float64), np.zeros(K, dtype=np.int32))
        outs.append(o)
        sp[i], lp[i], rp[i], np_[i] = (a.ctypes.data for a in o)
    hs = (ctypes.c_void_p * count)(*[L.h.value for L in learners])
    sc = None
    if scores is not None:
        assert shrinkage is not None and len(scores) == count
        sc = (ctypes.c_void_p * count)(*[int(s) for s in scores])
    _lib.check(lib.bk_learners_train_batch(hs, count, gp, hp, int(bool(on_device)),
                                           float(shrinkage if shrinkage is not None else 0.0), sc, sp, lp, rp, np_),
               "bk_learners_train_batch")
    return outs


class LearnerGroup:
    """A fixed set of learners whose iterations run as one CUDA graph (``bk_learner_group_*``):
    every learner's grow loop, score update and result readback is one branch of the graph, so one
    launch runs all of them with no host work between their kernels."""

    def __init__(self, learners):
        self.learners = list(learners)
        assert self.learners
        self.lib = self.learners[0].lib
        count = len(self.learners)
        hs = (ctypes.c_void_p * count)(*[L.h.value for L in self.learners])
        h = ctypes.c_void_p()
        _lib.check(self.lib.bk_learner_group_create(hs, count, ctypes.byref(h)), "bk_learner_group_create")
        self.h = h
        self._outs = []
        for L in self.learners:
            K, Lv = L.num_jobs, L.num_leaves
            self._outs.append((np.zeros((K, max(Lv - 1, 1)), dtype=SPLIT_DTYPE), np.zeros((K, Lv), dtype=np.float64),
                               np.zeros(K, dtype=np.float64), np.zeros(K, dtype=np.int32)))
        arr = lambda k: (ctypes.c_void_p * count)(*[o[k].ctypes.data for o in self._outs])
        self._sp, self._lp, self._rp, self._np = arr(0), arr(1), arr(2), arr(3)

    def train(self, gradients, hessians, shrinkage=0.0, scores=None):
        """One iteration of every learner: gradients / hessians are per learner device pointers
        ([num_jobs, num_data] f32); scores None or per learner a device f64 score pointer, which
        receives the new trees' leaf outputs times ``shrinkage``. Returns per learner (splits,
        leaf_values, root_outputs, num_leaves), arrays the next call overwrites."""
        count = len(self.learners)
        gp = (ctypes.c_void_p * count)(*[int(g) for g in gradients])
        hp = (ctypes.c_void_p * count)(*[int(x) for x in hessians])
        sc = None if scores is None else (ctypes.c_void_p * count)(*[int(s) for s in scores])
        _lib.check(self.lib.bk_learner_group_train(self.h, gp, hp, float(shrinkage), sc, self._sp, self._lp, self._rp,
                                                   self._np), "bk_learner_group_train")
        return self._outs

    def autotune(self, gradients, hessians, trials=2):
        """Picks the group's launch policy by timing whole group iterations
        (bk_learner_group_autotune); returns (launch overlap, rows per histogram CTA, histogram
        CTAs per member, partition CTAs)."""
        count = len(self.learners)
        gp = (ctypes.c_void_p * count)(*[int(g) for g in gradients])
        hp = (ctypes.c_void_p * count)(*[int(x) for x in hessians])
        out = np.zeros(4, np.int32)
        _lib.check(self.lib.bk_learner_group_autotune(self.h, gp, hp, int(trials), out.ctypes.data),
                   "bk_learner_group_autotune")
        return tuple(int(x) for x in out)

    def close(self):
        if self.h:
            self.lib.bk_learner_group_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

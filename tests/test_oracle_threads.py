"""Training must not depend on num_threads (crates/lgbm-core/tests/thread_invariance.rs:97-134):
the oracle grows identical trees (15 iterations, 31 leaves) with 1, 2 and 3 worker threads, on
the reference's own splitmix64 data generators (8,000 rows here instead of 40,000), for the
full-precision path and for the quantized path with nearest rounding (8 gradient bins). The GPU learner's trees are compared with the oracle's elsewhere, so this
pins that the oracle itself is thread-invariant, as the reference is.
"""
import numpy as np
import pytest

MASK = (1 << 64) - 1


def _splitmix(state):
    while True:
        state = (state + 0x9E3779B97F4A7C15) & MASK
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        yield z ^ (z >> 31)


def _synthetic(nrow, ncol, dense):
    """thread_invariance.rs:12-59: synthetic (every third column mostly zero) and dense_synthetic."""
    rnd = _splitmix(0x2545F4914F6CDD1D if dense else 0x9E3779B97F4A7C15)
    x = np.zeros((nrow, ncol))
    for r in range(nrow):
        for c in range(ncol):
            u = (next(rnd) >> 11) / float(1 << 53)
            if dense:
                x[r, c] = u * (c + 1.0) - 0.5
            else:
                x[r, c] = 0.0 if (c % 3 == 0 and u < 0.8) else u * (c + 1.0)
    y = x[:, 0] + 2.0 * x[:, 1] - x[:, 2] * x[:, 3]
    return x, y


def _trees(oracle, ds, y, threads, **extra):
    from lgbm_gb300 import LearnerConfig
    obj = oracle.make_objective({"objective": "regression"}, y)
    cfg = LearnerConfig(num_leaves=31, min_data_in_leaf=20, num_threads=threads, fused_madd=1,
                        is_constant_hessian=1, **extra)
    trees, _ = oracle.train_gbdt(oracle.OracleLearner(ds, cfg), ds, obj, 15)
    return trees


@pytest.mark.parametrize("quantized", [False, True])
def test_trees_independent_of_num_threads(oracle, bklib, quantized):
    from lgbm_gb300 import BinnedDataset
    nrow, ncol = (8000, 20) if quantized else (8000, 40)
    x, y = _synthetic(nrow, ncol, dense=quantized)
    ds = BinnedDataset.from_dense(x)
    extra = dict(use_quantized_grad=1, stochastic_rounding=0, num_grad_quant_bins=8) if quantized else {}
    serial = _trees(oracle, ds, y, 1, **extra)
    assert len(serial) == 15
    for threads in (2, 3):
        par = _trees(oracle, ds, y, threads, **extra)
        assert len(par) == len(serial)
        for a, b in zip(serial, par):
            assert a.num_leaves == b.num_leaves
            n = a.num_leaves - 1
            for name in ("split_feature", "threshold", "left_child", "right_child", "internal_count"):
                assert np.array_equal(getattr(a, name)[:n], getattr(b, name)[:n]), name
            assert np.array_equal(a.leaf_value[:a.num_leaves], b.leaf_value[:b.num_leaves])

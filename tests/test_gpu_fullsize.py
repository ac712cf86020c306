"""Parity at the benchmark's full size: one 255-leaf tree on 10,000,000 rows x 100 features
(the L2 step-function workload: 70 N(0,1) + 30 integer features, 10% NaN), grown by the GB300
learner and by the oracle on the same binned rows and the same gradients.

* quantized path (int8 stochastic-rounding gradients, integer histograms): every split record,
  every leaf value and the row -> leaf partition of all 10M rows equal the oracle's bit for bit;
* float path: the same tree structure and every split gain within 1e-6 relative (near-tie
  divergences counted, at most one allowed).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROWS = 10_000_000


@pytest.fixture(scope="module")
def workload():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lgbm_gb300 import BinnedDataset, synthetic
    X, y = synthetic.l2_steps(n=ROWS, seed=0)
    threads = min(32, os.cpu_count() or 8)
    ds = BinnedDataset.from_dense(X, max_bin=255, min_data_in_leaf=20, threads=threads)
    del X
    # the first boosting iteration's L2 gradients from the boost-from-average score
    g = (np.float64(np.mean(y, dtype=np.float64)) - y.astype(np.float64)).astype(np.float32)
    return ds, g, threads


def _learners(ds, quant, threads):
    import harness
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig
    cfg = LearnerConfig(num_leaves=255, min_data_in_leaf=20, use_quantized_grad=quant, num_grad_quant_bins=4,
                        stochastic_rounding=1, seed=0, num_threads=threads, fused_madd=1, is_constant_hessian=1)
    return harness.OracleLearner(ds, cfg), GpuTreeLearner(ds, cfg, loop_mode=1)


def test_quantized_tree_bit_exact_at_full_size(workload):
    ds, g, threads = workload
    h = np.ones_like(g)
    orc, gpu = _learners(ds, 1, threads)
    ro, rg = orc.train(g, h), gpu.train(g, h)
    assert len(rg[0]) == 254, "a 255-leaf tree"
    assert len(ro[0]) == len(rg[0])
    for name in ro[0].dtype.names:
        a, b = ro[0][name], rg[0][name]
        assert np.array_equal(a, b), "split field %s differs at split %d" % (name, int(np.flatnonzero(a != b)[0]))
    assert np.array_equal(ro[1], rg[1])
    assert ro[2] == rg[2]
    assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
    gpu.close()


def test_float_tree_matches_at_full_size(workload):
    ds, g, threads = workload
    h = np.ones_like(g)
    orc, gpu = _learners(ds, 0, threads)
    ro, rg = orc.train(g, h), gpu.train(g, h)
    # the whole tree, past any near tie: nodes keyed by their root path, gains of matched nodes
    # within 1e-6 relative, divergences counted, listed and bounded
    import harness
    m = harness.split_match(rg[0], ro[0])
    print("float tree vs oracle: %d matched, %d diverged, max rel gain error %.3g, mean %.3g"
          % (m["matched"], m["diverged"], m["max_rel"], m["mean_rel"]))
    for d in m["divergences"]:
        print("  divergence:", d)
    assert m["max_rel"] <= 1e-6, m
    assert m["matched"] >= 0.8 * max(len(ro[0]), len(rg[0])), m
    gpu.close()

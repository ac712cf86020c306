"""The device kernels around the learner, each against its reference computation:

* objective gradients (bk_learner_objective_gradients): L2 (objective/regression.rs:240-248)
  bit for bit; binary (objective/binary.rs:71-90) and softmax (objective/multiclass.rs:68-90)
  within one f32 ulp (CUDA's exp against the host's, in the last f64 bit), in the reference's
  operation order; with row weights (regression.rs:321-329 for L2, bit for bit) and the binary
  label weights of is_unbalance / scale_pos_weight (binary.rs:33-52) against the oracle harness's
  weighted objectives; a multiclass label outside [0, K) fails the next train call and the loss
  call instead of indexing the scores;
* held-out prediction (bk_learner_predict_add, the replay of serial.rs:2009-2041) on upstream's own
  models and test rows (tests/fixtures/predict: binary, NaN, zero as missing, L2, a categorical
  feature (bin bitsets), 3-class): every
  row reaches upstream's leaf in every tree (pred_leaf.npy) and the raw scores, the leaf values
  added in tree order on the device, equal upstream's bit for bit (pred_raw.npy).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

PREDICT = os.path.join(GOLDEN, "predict")
PREDICT_CASES = ["binary", "categorical", "missing", "multiclass", "regression_l2", "zero_as_missing"]


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _ulps(a, b):
    """Distance in f32 units in the last place (same-sign finite values)."""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(ia - ib)


def _grads_host(kind, score, label, K):
    """The reference's gradient formulas, vectorized in the reference's operation order."""
    if kind == 0:
        return (score - label.astype(np.float64)).astype(np.float32), np.ones_like(label, dtype=np.float32)
    if kind == 1:
        lab = np.where(label > 0, 1.0, -1.0)
        response = (-lab * 1.0) / (1.0 + np.exp(lab * 1.0 * score))
        ar = np.abs(response)
        return (response * 1.0).astype(np.float32), ((ar * (1.0 - ar)) * 1.0).astype(np.float32)
    s = score.reshape(K, -1)
    wmax = s[0].copy()
    for k in range(1, K):
        wmax = np.fmax(s[k], wmax)
    rec = np.exp(s - wmax)
    wsum = np.zeros_like(wmax)
    for k in range(K):
        wsum += rec[k]
    p = rec / wsum
    lab = label.astype(np.int64)
    g = p - (np.arange(K)[:, None] == lab[None, :])
    h = (K / (K - 1.0)) * p * (1.0 - p)
    return g.astype(np.float32), h.astype(np.float32)


def _device_grads(kind, score_np, label_np, K, n):
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    rng = np.random.default_rng(0)
    ds = BinnedDataset.from_dense(rng.standard_normal((n, 3)))
    gpu = GpuTreeLearner(ds, LearnerConfig(num_leaves=4), num_jobs=K)
    score = torch.from_numpy(score_np).cuda()
    label = torch.from_numpy(label_np).cuda()
    torch.cuda.synchronize()
    gpu.objective_gradients(kind, score.data_ptr(), label.data_ptr())
    gp, hp = gpu.gradient_buffers()
    g = torch.empty(K * n, dtype=torch.float32, device="cuda")
    h = torch.empty(K * n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(gpu.stream())
    with torch.cuda.stream(stream):
        g.copy_(_view(gp, K * n))
        h.copy_(_view(hp, K * n))
    stream.synchronize()
    return gpu, score, label, g.cpu().numpy().reshape(K, n), h.cpu().numpy().reshape(K, n)


def _view(ptr, count):
    import torch

    class _CAI:
        __cuda_array_interface__ = {"shape": (count,), "typestr": "<f4", "data": (int(ptr), False), "version": 3,
                                    "strides": None}
    return torch.as_tensor(_CAI(), device="cuda")


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_objective_gradients_on_device(oracle, kind):
    n = 300_000
    K = 7 if kind == 2 else 1
    rng = np.random.default_rng(kind)
    score = rng.normal(0.0, 2.0, K * n)
    if kind == 0:
        label = rng.normal(0.0, 3.0, n).astype(np.float32)
    elif kind == 1:
        label = (rng.random(n) < 0.4).astype(np.float32)
    else:
        label = rng.integers(0, K, n).astype(np.float32)
    gpu, _, _, g, h = _device_grads(kind, score, label, K, n)
    gw, hw = _grads_host(kind, score, label, K)
    gw, hw = gw.reshape(K, n), hw.reshape(K, n)
    if kind == 0:
        assert np.array_equal(g, gw) and np.array_equal(h, hw)
    else:
        assert int(_ulps(g, gw).max()) <= 1 and int(_ulps(h, hw).max()) <= 1
        print("rows off by one ulp: g %d, h %d of %d" % (int((g != gw).sum()), int((h != hw).sum()), g.size))
    # the vectorized formulas above against the oracle harness's per-row restatement (first rows)
    m = 500
    if kind == 1:
        go, ho = oracle.BinaryObjective(label[:m]).gradients(score[:m])
    elif kind == 2:
        go, ho = oracle.SoftmaxObjective(label[:m], K).gradients(score.reshape(K, n)[:, :m])
    else:
        go = (score[:m] - label[:m].astype(np.float64)).astype(np.float32)[None, :]
        ho = np.ones((1, m), np.float32)
    assert int(_ulps(go, gw[:, :m]).max()) <= 1 and int(_ulps(ho, hw[:, :m]).max()) <= 1
    gpu.close()


@pytest.mark.parametrize("kind,weighted,is_unbalance,scale_pos", [
    (0, True, False, 1.0), (1, True, False, 1.0), (1, False, True, 1.0), (1, False, False, 2.5),
    (1, True, True, 1.0), (2, True, False, 1.0)])
def test_weighted_objective_gradients_on_device(oracle, kind, weighted, is_unbalance, scale_pos):
    """Row weights and binary label weights (bk_learner_set_objective_weights) against the oracle
    harness's weighted objectives: L2 bit for bit, binary / softmax within one f32 ulp."""
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    n = 4000
    K = 4 if kind == 2 else 1
    rng = np.random.default_rng(40 + kind)
    score = rng.normal(0.0, 1.5, (K, n))
    if kind == 0:
        label = rng.normal(0.0, 2.0, n).astype(np.float32)
    elif kind == 1:
        label = (rng.random(n) < 0.3).astype(np.float32)
    else:
        label = rng.integers(0, K, n).astype(np.float32)
    w = rng.uniform(0.2, 3.0, n).astype(np.float32) if weighted else None
    if kind == 0:
        obj = oracle.L2Objective(label, weights=w)
    elif kind == 1:
        obj = oracle.BinaryObjective(label, weights=w, is_unbalance=is_unbalance, scale_pos_weight=scale_pos)
    else:
        obj = oracle.SoftmaxObjective(label, K, weights=w)
    go, ho = obj.gradients(score if kind == 2 else score[0])
    go, ho = np.asarray(go).reshape(K, n), np.asarray(ho).reshape(K, n)
    ds = BinnedDataset.from_dense(rng.standard_normal((n, 3)))
    gpu = GpuTreeLearner(ds, LearnerConfig(num_leaves=4), num_jobs=K)
    sc = torch.from_numpy(np.ascontiguousarray(score.reshape(-1))).cuda()
    lab = torch.from_numpy(label).cuda()
    wd = torch.from_numpy(w).cuda() if weighted else None
    lw = obj.label_weights if kind == 1 else [1.0, 1.0]
    torch.cuda.synchronize()
    gpu.set_objective_weights(wd.data_ptr() if weighted else 0, lw[0], lw[1])
    gpu.objective_gradients(kind, sc.data_ptr(), lab.data_ptr())
    gp, hp = gpu.gradient_buffers()
    stream = torch.cuda.ExternalStream(gpu.stream())
    with torch.cuda.stream(stream):
        g = _view(gp, K * n).clone()
        h = _view(hp, K * n).clone()
    stream.synchronize()
    g, h = g.cpu().numpy().reshape(K, n), h.cpu().numpy().reshape(K, n)
    if kind == 0:
        assert np.array_equal(g, go) and np.array_equal(h, ho)
    else:
        assert int(_ulps(g, go).max()) <= 1 and int(_ulps(h, ho).max()) <= 1
    # weights off again: the unweighted formulas
    gpu.set_objective_weights(0, 1.0, 1.0)
    gpu.objective_gradients(kind, sc.data_ptr(), lab.data_ptr())
    with torch.cuda.stream(stream):
        g2 = _view(gp, K * n).clone()
    stream.synchronize()
    gu, _ = _grads_host(kind, score.reshape(-1), label, K)
    assert int(_ulps(g2.cpu().numpy().reshape(K, n), gu.reshape(K, n)).max()) <= 1
    with pytest.raises(RuntimeError):
        gpu.set_objective_weights(0, 0.0, 1.0)
    gpu.close()


def test_bad_multiclass_label_is_an_error():
    """A label outside [0, K) is never used as an index: the next train call and the loss fail."""
    import torch
    n, K = 20000, 3
    rng = np.random.default_rng(9)
    score = rng.normal(0, 1, K * n)
    label = rng.integers(0, K, n).astype(np.float32)
    label[123] = K  # not a class
    label[77] = np.nan
    gpu, sc, lab, g, h = _device_grads(2, score, label, K, n)
    gp, hp = gpu.gradient_buffers()
    with pytest.raises(RuntimeError, match="labels outside"):
        gpu.train_raw(gp, hp, on_device=True)
    with pytest.raises(RuntimeError, match="labels outside"):
        gpu.objective_loss(2, sc.data_ptr(), lab.data_ptr())
    # the next iteration on valid labels works again
    lab.copy_(torch.from_numpy(np.clip(np.nan_to_num(label), 0, K - 1)).cuda())
    torch.cuda.synchronize()
    gpu.objective_gradients(2, sc.data_ptr(), lab.data_ptr())
    gpu.train_raw(gp, hp, on_device=True)
    assert np.isfinite(gpu.objective_loss(2, sc.data_ptr(), lab.data_ptr()))
    gpu.close()


@pytest.mark.parametrize("case", PREDICT_CASES)
def test_device_prediction_matches_upstream(oracle, bklib, case):
    import torch
    from test_route_golden import _Tree
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    d = os.path.join(PREDICT, case)
    P = json.load(open(os.path.join(d, "params.json")))
    train = np.load(os.path.join(d, "train.npy"))
    test = np.load(os.path.join(d, "test.npy"))
    want_leaf = np.load(os.path.join(d, "pred_leaf.npy"))
    raw_want = np.load(os.path.join(d, "pred_raw.npy")).reshape(len(test), -1)
    ds = BinnedDataset.from_dense(train[:, 1:], zero_as_missing=P["params"].get("zero_as_missing", False),
                                  categorical=P["dataset"].get("categorical_feature", []))
    held = torch.from_numpy(np.ascontiguousarray(ds.bin_like(test[:, 1:]))).cuda()
    trees = oracle.parse_model_trees(open(os.path.join(d, "model.txt")).read())
    max_leaves = max(int(rec["num_leaves"]) for rec in trees)
    gpu = GpuTreeLearner(ds, LearnerConfig(num_leaves=max(max_leaves, 2)))
    m, K = len(test), raw_want.shape[1]
    raw = torch.zeros((K, m), dtype=torch.float64, device="cuda")
    for k, rec in enumerate(trees):
        t = _Tree(rec, ds)
        t.leaf_value = np.array([float(v) for v in rec["leaf_value"].split()])
        # the leaf each row reaches: leaf values 0, 1, 2, ... added to a zero score
        idx = torch.zeros(m, dtype=torch.float64, device="cuda")
        probe = _Tree(rec, ds)
        probe.leaf_value = np.arange(t.num_leaves, dtype=np.float64)
        torch.cuda.synchronize()
        gpu.predict_add(probe, held.data_ptr(), m, idx.data_ptr())
        got = idx.cpu().numpy().astype(np.int64)
        assert np.array_equal(got, want_leaf[:, k]), "tree %d: %d rows differ" % (k, int((got != want_leaf[:, k]).sum()))
        gpu.predict_add(t, held.data_ptr(), m, raw[k % K].data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(raw.cpu().numpy().T, raw_want), "raw scores differ"
    gpu.close()

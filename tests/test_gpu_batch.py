"""Many independent boosting jobs in one call (bk_learners_train_batch): learners with different
row counts, feature counts, max_bin and configs, each on its own stream, queued together.

Every quantized tree grown in the batch equals the oracle's tree for the same job bit for bit
(split records, leaf values, partition); a float job matches within the float tolerance; and the
device score update applied by the batch equals the host update with the returned leaf values
(shrinkage 0.1, Tree::apply_shrinkage rounding).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (rows, features, max_bin, quantized)
JOBS = [(5000, 20, 15, 1), (23000, 45, 63, 1), (61000, 100, 255, 1), (12000, 300, 255, 1), (40000, 33, 15, 1),
        (30000, 64, 63, 0)]


def _job(i, n, F, max_bin):
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(100 + i)
    X = rng.standard_normal((n, F))
    X[rng.random((n, F)) < 0.01] = np.nan
    w = rng.standard_normal(F) * (rng.random(F) < 0.3)
    z = np.nan_to_num(X) @ w
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-z))).astype(np.float64)
    return BinnedDataset.from_dense(X, max_bin=max_bin), y


def _binary_grads(score, y):
    p = 1.0 / (1.0 + np.exp(-score))
    return (p - y).astype(np.float32), (p * (1.0 - p)).astype(np.float32)


def _round0(v):
    v = v.copy()
    v[np.abs(v) <= float(np.float32(1e-35))] = 0.0
    return v


def test_batch_of_independent_jobs_matches_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import harness
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig, train_batch
    jobs = []
    for i, (n, F, mb, quant) in enumerate(JOBS):
        ds, y = _job(i, n, F, mb)
        cfg = LearnerConfig(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=i, num_threads=2)
        score = np.zeros(n)
        dscore = torch.zeros(n, dtype=torch.float64, device="cuda")
        jobs.append(dict(ds=ds, y=y, gpu=GpuTreeLearner(ds, cfg), orc=harness.OracleLearner(ds, cfg), score=score,
                         dscore=dscore, quant=quant))
    torch.cuda.synchronize()
    float_divergences = []  # near-tie split choices of the float job (at most one tree allowed)
    for it in range(3):
        grads = [_binary_grads(j["score"], j["y"]) for j in jobs]
        outs = train_batch([j["gpu"] for j in jobs], [g for g, _ in grads], [h for _, h in grads], shrinkage=0.1,
                           scores=[j["dscore"].data_ptr() for j in jobs])
        for j, (g, h), (splits, lv, roots, nls) in zip(jobs, grads, outs):
            nl = int(nls[0])
            ro = j["orc"].train(g, h)
            if j["quant"]:
                assert len(ro[0]) == nl - 1
                for name in ro[0].dtype.names:
                    assert np.array_equal(ro[0][name], splits[0, :nl - 1][name]), (it, name)
                assert np.array_equal(ro[1], lv[0, :nl])
                assert np.array_equal(j["orc"].row_leaf(), j["gpu"].row_leaf())
            else:
                a, b = ro[0], splits[0, :nl - 1]
                same = len(a) == len(b) and all(a[k]["threshold"] == b[k]["threshold"] and
                                                a[k]["real_feature"] == b[k]["real_feature"] for k in range(len(a)))
                if same:
                    assert np.allclose(a["gain"], b["gain"], rtol=1e-6, atol=0)
                else:
                    float_divergences.append(it)
            if nl > 1:
                j["score"] += _round0(lv[0, :nl] * 0.1)[j["gpu"].row_leaf()]
            assert np.array_equal(j["dscore"].cpu().numpy(), j["score"]), "device score update, iteration %d" % it
    print("float near-tie divergences (iterations):", float_divergences)
    assert len(float_divergences) <= 1
    for j in jobs:
        j["gpu"].close()


def test_batch_rejects_a_learner_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig, train_batch
    ds, y = _job(0, 3000, 10, 63)
    gpu = GpuTreeLearner(ds, LearnerConfig(num_leaves=7))
    g, h = _binary_grads(np.zeros(len(y)), y)
    with pytest.raises(RuntimeError, match="appears twice"):
        train_batch([gpu, gpu], [g, g], [h, h])
    gpu.close()


def test_learner_group_matches_oracle():
    """The same jobs as one CUDA graph (bk_learner_group_*), after the group's launch-policy
    autotuner: every quantized tree equals the oracle's bit for bit, the float job's within the
    float tolerance, the device score update the host's; changing one member's launch shape
    recaptures the graph and changes no result."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import harness
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig, LearnerGroup
    jobs = []
    for i, (n, F, mb, quant) in enumerate(JOBS):
        ds, y = _job(i, n, F, mb)
        cfg = LearnerConfig(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=i, num_threads=2)
        jobs.append(dict(ds=ds, y=y, gpu=GpuTreeLearner(ds, cfg), orc=harness.OracleLearner(ds, cfg),
                         score=np.zeros(n), dscore=torch.zeros(n, dtype=torch.float64, device="cuda"),
                         dg=torch.zeros(n, dtype=torch.float32, device="cuda"),
                         dh=torch.zeros(n, dtype=torch.float32, device="cuda"), quant=quant))
    group = LearnerGroup([j["gpu"] for j in jobs])
    # the launch-policy autotuner first: its trial iterations must leave every learner's state
    # (the stochastic-rounding engines) as it found it, so the trees below still equal the oracle's
    for j in jobs:
        g0, h0 = _binary_grads(j["score"], j["y"])
        j["dg"].copy_(torch.from_numpy(g0))
        j["dh"].copy_(torch.from_numpy(h0))
    torch.cuda.synchronize()
    policy = group.autotune([j["dg"].data_ptr() for j in jobs], [j["dh"].data_ptr() for j in jobs], trials=1)
    assert policy[0] in (0, 1) and policy[2] in (38, 19, 10, 5), policy
    float_divergences = []
    for it in range(4):
        if it == 2:
            jobs[2]["gpu"].set_launch_shape((64, 7, 40, 0))  # the group graph is captured anew
        grads = [_binary_grads(j["score"], j["y"]) for j in jobs]
        for j, (g, h) in zip(jobs, grads):
            j["dg"].copy_(torch.from_numpy(g))
            j["dh"].copy_(torch.from_numpy(h))
        torch.cuda.synchronize()
        outs = group.train([j["dg"].data_ptr() for j in jobs], [j["dh"].data_ptr() for j in jobs], shrinkage=0.1,
                           scores=[j["dscore"].data_ptr() for j in jobs])
        for j, (g, h), (splits, lv, roots, nls) in zip(jobs, grads, outs):
            nl = int(nls[0])
            ro = j["orc"].train(g, h)
            if j["quant"]:
                assert len(ro[0]) == nl - 1
                for name in ro[0].dtype.names:
                    assert np.array_equal(ro[0][name], splits[0, :nl - 1][name]), (it, name)
                assert np.array_equal(ro[1], lv[0, :nl])
                assert np.array_equal(j["orc"].row_leaf(), j["gpu"].row_leaf())
            else:
                m = harness.split_match(splits[0, :nl - 1], ro[0])
                assert m["max_rel"] <= 1e-6, m
                if m["diverged"]:
                    float_divergences.append(it)
            if nl > 1:
                j["score"] += _round0(lv[0, :nl] * 0.1)[j["gpu"].row_leaf()]
            assert np.array_equal(j["dscore"].cpu().numpy(), j["score"]), "device score update, iteration %d" % it
    print("float near-tie divergences (iterations):", float_divergences)
    assert len(float_divergences) <= 1
    group.close()
    for j in jobs:
        j["gpu"].close()

"""Parity at the full sizes of the benchmark's other workloads, GB300 learner against the oracle on
the same binned rows and the same gradients:

* binary, 10,000,000 rows x 200 features (100 N(0,1) + 100 uniform(-1, 1), 5% NaN, sparse
  logistic labels; the rows the benchmark's binary form trains on), varying hessians from device
  binary gradients, 4 gradient bins with stochastic rounding, 255 leaves: every split record, leaf
  value, the root output and the row -> leaf map of all 10M rows bit for bit
  (serial.rs:1074-1164, gradient_discretizer/mod.rs:172-201);
* multiclass softmax K = 10, 2,000,000 x 64 Gaussian mixture, max_bin 63, 63 leaves: one iteration
  of all ten class trees grown in one call, quantized bit for bit against ten sequential oracle
  trees (one shared discretizer), float within 1e-6 relative gains with near-tie divergences
  counted and listed;
* the 256 independent jobs of the batched workload (rows 5k-500k, 20-300 features, max_bin 15 / 63
  / 255, 31 leaves), all grown in one bk_learners_train_batch call: every quantized tree bit for
  bit against the oracle's.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = min(32, os.cpu_count() or 8)


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _assert_same_tree(ro, rg_splits, rg_values, rg_root=None):
    assert len(ro[0]) == len(rg_splits), "splits %d vs %d" % (len(ro[0]), len(rg_splits))
    for name in ro[0].dtype.names:
        a, b = ro[0][name], rg_splits[name]
        assert np.array_equal(a, b), "field %s differs at split %d" % (name, int(np.flatnonzero(
            np.any(a != b, axis=tuple(range(1, a.ndim))) if a.ndim > 1 else a != b)[0]))
    assert np.array_equal(ro[1], rg_values)
    if rg_root is not None:
        assert ro[2] == rg_root


def test_binary_10M_x_200_quantized_tree_bit_exact(oracle):
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    rows, F = 10_000_000, 200
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    X = torch.empty((rows, F), dtype=torch.float32, device="cuda")
    X[:, :F // 2].normal_(generator=gen)
    X[:, F // 2:].uniform_(-1.0, 1.0, generator=gen)
    w = torch.zeros(F, dtype=torch.float32, device="cuda")
    nz = torch.randperm(F, generator=gen, device="cuda")[:F // 10]
    w[nz] = torch.randn(F // 10, generator=gen, device="cuda")
    y = (torch.rand(rows, generator=gen, device="cuda") < torch.sigmoid(X @ w)).float()
    for c0 in range(0, F, 25):
        blk = X[:, c0:c0 + 25]
        blk[torch.rand(blk.shape, generator=gen, device="cuda") < 0.05] = float("nan")
    ds = BinnedDataset.from_dense_device(X, max_bin=255, min_data_in_leaf=20, threads=THREADS)
    del X
    torch.cuda.empty_cache()
    host = BinnedDataset(ds.bins.cpu().numpy(), ds.features, ds.num_total_features)
    cfg = LearnerConfig(num_leaves=255, min_data_in_leaf=20, use_quantized_grad=1, num_grad_quant_bins=4,
                        stochastic_rounding=1, seed=0, num_threads=16, fused_madd=1)
    gpu = GpuTreeLearner(ds, cfg)
    # varying hessians: binary gradients (device kernel) at a perturbed boost-from-average score
    pavg = float(y.mean().item())
    score = torch.full((rows,), np.log(pavg / (1 - pavg)), dtype=torch.float64, device="cuda")
    score += 0.5 * torch.randn(rows, generator=gen, device="cuda", dtype=torch.float64)
    torch.cuda.synchronize()
    gpu.objective_gradients(1, score.data_ptr(), y.data_ptr())
    gp, hp = gpu.gradient_buffers()
    stream = torch.cuda.ExternalStream(gpu.stream())
    from test_gpu_device_kernels import _view
    with torch.cuda.stream(stream):
        g = _view(gp, rows).cpu().numpy()
        h = _view(hp, rows).cpu().numpy()
    assert np.unique(h[:100000]).size > 100, "the hessians vary"
    orc = oracle.OracleLearner(host, cfg)
    orc.set_threads(THREADS)
    ro = orc.train(g, h)
    sp, lv, roots, nls = gpu.train_raw(g[None, :], h[None, :])
    assert nls[0] == 255
    _assert_same_tree(ro, sp[0, :nls[0] - 1], lv[0, :nls[0]], roots[0])
    assert np.array_equal(orc.row_leaf(), gpu.row_leaf())
    gpu.close()


def _mixture(oracle):
    from lgbm_gb300 import BinnedDataset, synthetic
    X, y = synthetic.gaussian_mixture(n=2_000_000, F=64, K=10, seed=0)
    ds = BinnedDataset.from_dense(X, max_bin=63, min_data_in_leaf=20, threads=THREADS)
    K, n = 10, ds.num_data
    prior = np.bincount(y.astype(np.int64), minlength=K) / float(n)
    rng = np.random.default_rng(4)
    score = np.log(np.maximum(prior, 1e-15))[:, None] + rng.normal(0.0, 0.3, (K, n))
    # softmax gradients (objective/multiclass.rs:68-90), vectorized in the reference's order
    from test_gpu_device_kernels import _grads_host
    g, h = _grads_host(2, score.ravel(), y, K)
    return ds, g.reshape(K, n), h.reshape(K, n)


@pytest.mark.parametrize("quant", [1, 0])
def test_multiclass_k10_iteration(oracle, quant):
    from lgbm_gb300 import GpuTreeLearner, LearnerConfig
    ds, G, H = _mixture(oracle)
    K = 10
    cfg = LearnerConfig(num_leaves=63, min_data_in_leaf=20, use_quantized_grad=quant, num_grad_quant_bins=4,
                        stochastic_rounding=1, seed=0, num_threads=16, fused_madd=1)
    gpu = GpuTreeLearner(ds, cfg, num_jobs=K)
    orc = oracle.OracleLearner(ds, cfg)
    orc.set_threads(THREADS)
    sp, lv, roots, nls = gpu.train_raw(G, H)
    rl = gpu.row_leaf() if quant else None
    divergences, worst = [], 0.0
    for k in range(K):
        ro = orc.train(G[k], H[k])
        if quant:
            _assert_same_tree(ro, sp[k, :nls[k] - 1], lv[k, :nls[k]], roots[k])
            assert np.array_equal(orc.row_leaf(), rl[k])
            continue
        errs = oracle.gain_errors(sp[k, :nls[k] - 1], ro[0])
        worst = max(worst, errs["max_rel"])
        assert errs["max_rel"] <= 1e-6, (k, errs)
        if errs["near_ties"]:
            divergences.append((k, errs["near_ties"][0]))
        else:
            assert nls[k] - 1 == len(ro[0])
    if not quant:
        print("float K=10: max gain rel error %.3g; near-tie divergences: %s" % (worst, divergences))
        assert len(divergences) <= 3
    gpu.close()


def test_batched_jobs_256_shapes_quantized_bit_exact(oracle):
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig, synthetic, train_batch
    jobs = []
    for i, (X, y, mb) in enumerate(synthetic.batched_jobs(256, seed=7)):
        ds = BinnedDataset.from_dense(X, max_bin=mb, min_data_in_leaf=20, threads=THREADS)
        rng = np.random.default_rng(1000 + i)
        score = rng.normal(0.0, 0.5, ds.num_data)
        p = 1.0 / (1.0 + np.exp(-score))
        g = (p - y).astype(np.float32)
        h = (p * (1.0 - p)).astype(np.float32)
        cfg = LearnerConfig(num_leaves=31, min_data_in_leaf=20, use_quantized_grad=1, num_grad_quant_bins=4,
                            stochastic_rounding=1, seed=i, num_threads=16, fused_madd=1)
        jobs.append((ds, cfg, g, h))
    assert len(jobs) == 256
    learners = [GpuTreeLearner(ds, cfg) for ds, cfg, _, _ in jobs]
    torch.cuda.synchronize()
    outs = train_batch(learners, [j[2] for j in jobs], [j[3] for j in jobs])
    bins_seen = set()
    for i, ((ds, cfg, g, h), (sp, lv, roots, nls), L) in enumerate(zip(jobs, outs, learners)):
        orc = oracle.OracleLearner(ds, cfg)
        orc.set_threads(THREADS)
        ro = orc.train(g, h)
        _assert_same_tree(ro, sp[0, :nls[0] - 1], lv[0, :nls[0]], roots[0])
        assert np.array_equal(orc.row_leaf(), L.row_leaf()), "job %d partition" % i
        bins_seen.add(max(fi.num_bin for fi in ds.features))
        L.close()
    assert len(bins_seen) >= 3

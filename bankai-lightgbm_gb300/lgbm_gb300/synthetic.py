"""Seeded synthetic datasets with the shapes and value distributions of the benchmark
workloads (the public datasets the reference mentions are not available, so these stand in):

* ``higgs_like``   — binary, 21 correlated N(0,1) features + 7 derived (products / abs), labels
  from a logistic model with 3 pairwise interactions (100k x 28);
* ``l2_steps``     — L2 regression, 70 N(0,1) + 30 integer 0..15 features, 10% NaN, target = sum
  of 20 random step functions + N(0, 0.1) noise (10M x 100);
* ``binary_sparse_linear`` — binary, N(0,1) / uniform mix, 5% NaN, labels from a sparse linear
  logistic model (10M x 200);
* ``gaussian_mixture`` — 10-class mixture with unit covariance and means spread 2.0 (2M x 64).

Every generator takes the row / feature counts so tests can use small instances.
"""
import numpy as np


def _nan_mask(rng, X, frac):
    if frac > 0:
        m = rng.random(X.shape, dtype=np.float32) < frac
        X[m] = np.nan
    return X


def higgs_like(n=100_000, seed=0):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((n, 1), dtype=np.float32)
    e = rng.standard_normal((n, 21), dtype=np.float32)
    base = np.sqrt(0.3).astype(np.float32) * c + np.sqrt(0.7).astype(np.float32) * e
    pairs = rng.integers(0, 21, size=(7, 2))
    derived = np.empty((n, 7), np.float32)
    for k, (a, b) in enumerate(pairs):
        derived[:, k] = base[:, a] * base[:, b] if k % 2 == 0 else np.abs(base[:, a])
    X = np.concatenate([base, derived], axis=1)
    w = rng.standard_normal(28).astype(np.float32) * 0.5
    z = X @ w
    for a, b in rng.integers(0, 28, size=(3, 2)):
        z += X[:, a] * X[:, b]
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-z))).astype(np.float32)
    return X, y


def l2_steps(n=10_000_000, n_cont=70, n_int=30, nan_frac=0.10, seed=0, nan_seed=1):
    rng = np.random.default_rng(seed)
    F = n_cont + n_int
    X = np.empty((n, F), np.float32)
    X[:, :n_cont] = rng.standard_normal((n, n_cont), dtype=np.float32)
    X[:, n_cont:] = rng.integers(0, 16, size=(n, n_int)).astype(np.float32)
    y = np.zeros(n, np.float32)
    for _ in range(20):
        f = int(rng.integers(0, F))
        col = np.nan_to_num(X[:, f], nan=0.0)
        thr = float(np.median(col[:10000])) + float(rng.standard_normal()) * 0.5
        y += np.where(col > thr, rng.standard_normal(), rng.standard_normal()).astype(np.float32)
    y += rng.normal(0.0, 0.1, n).astype(np.float32)
    _nan_mask(np.random.default_rng(nan_seed), X, nan_frac)
    return X, y


def binary_sparse_linear(n=10_000_000, F=200, nan_frac=0.05, seed=0):
    rng = np.random.default_rng(seed)
    X = np.empty((n, F), np.float32)
    half = F // 2
    X[:, :half] = rng.standard_normal((n, half), dtype=np.float32)
    X[:, half:] = rng.random((n, F - half), dtype=np.float32) * 2.0 - 1.0
    w = np.zeros(F, np.float32)
    nz = rng.choice(F, size=max(1, F // 10), replace=False)
    w[nz] = rng.standard_normal(len(nz)).astype(np.float32)
    z = X @ w
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-z))).astype(np.float32)
    _nan_mask(rng, X, nan_frac)
    return X, y


def gaussian_mixture(n=2_000_000, F=64, K=10, spread=2.0, seed=0):
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((K, F)).astype(np.float32) * spread / np.sqrt(F).astype(np.float32) * 4.0
    y = rng.integers(0, K, size=n)
    X = rng.standard_normal((n, F), dtype=np.float32) + means[y]
    return X, y.astype(np.float32)


def batched_jobs(count=256, seed=7):
    """The independent binary jobs of the batched workload, one at a time: rows log-uniform in
    [5,000, 500,000], features uniform in [20, 300] (N(0,1), 1% NaN), logistic labels from a per-job
    random linear model (20% of the weights non-zero), max_bin drawn from {15, 63, 255}. Yields
    (X float32 [rows, F], y float32 [rows], max_bin); one generator draws every job in order, so
    job i is the same however many jobs are taken."""
    rng = np.random.default_rng(seed)
    for _ in range(count):
        n = int(round(np.exp(rng.uniform(np.log(5_000), np.log(500_000)))))
        F = int(rng.integers(20, 301))
        mb = int(rng.choice([15, 63, 255]))
        X = rng.standard_normal((n, F), dtype=np.float32)
        w = (rng.standard_normal(F) * (rng.random(F) < 0.2)).astype(np.float32)
        z = X @ w
        X[rng.random((n, F), dtype=np.float32) < 0.01] = np.nan
        y = (rng.random(n) < 1.0 / (1.0 + np.exp(-z))).astype(np.float32)
        yield X, y, mb

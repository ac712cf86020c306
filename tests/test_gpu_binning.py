"""Device bin construction (bk_bin_dense_device) against two CPU references on the same values:

* a numpy restatement of BinMapper::value_to_bin (io/bin.rs:558-589: the first upper bound >= v,
  NaN to the NaN bin or to 0.0) and fill_dense (io/dataset.rs:633-685: the most frequent bin
  stored as 0, the others shifted past it);
* the host binning of BinnedDataset.from_dense, whose bins reproduce the reference's golden models
  (test_oracle_golden.py).

Stored bins are integers: equality is exact. Learners built from device bins must grow the same
trees as learners built from host bins.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _values(n, ncol, seed, dtype):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, ncol))
    X[:, 0] = 3.25  # constant: a trivial feature, dropped
    X[:, 1] = rng.integers(0, 16, n)
    X[:, 2] = np.where(rng.random(n) < 0.8, 0.0, rng.standard_normal(n))  # zero-heavy
    X[:, 3] = -np.abs(X[:, 3])  # all non-positive
    X[rng.random((n, ncol)) < 0.07] = np.nan
    X[:, 4] = np.where(rng.random(n) < 0.5, np.nan, X[:, 4])  # NaN-heavy
    X[:, 5] = rng.integers(-3, 4, n) * 0.5
    return X.astype(dtype)


def _numpy_stored_bins(X, features):
    """value_to_bin + fill_dense restated with numpy."""
    out = np.zeros((len(features), X.shape[0]), dtype=np.uint8)
    for j, fi in enumerate(features):
        v = X[:, fi.real].astype(np.float64)
        nan = np.isnan(v)
        rr = fi.num_bin - 1 - (1 if fi.missing_type == 2 else 0)
        b = np.searchsorted(fi.upper_bounds[:rr], np.where(nan, 0.0, v), side="left")
        if fi.missing_type == 2:
            b = np.where(nan, fi.num_bin - 1, b)
        mfb = fi.most_freq_bin
        out[j] = np.where(b == mfb, 0, b + 1 - (1 if mfb == 0 else 0)).astype(np.uint8)
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,ncol,max_bin,zam", [(20011, 24, 255, False), (3001, 300, 63, False),
                                                (5000, 12, 15, True), (1, 8, 255, False)])
def test_device_bins_match_host_and_numpy(dtype, n, ncol, max_bin, zam):
    import torch
    from lgbm_gb300 import BinnedDataset
    X = _values(n, ncol, seed=n + ncol, dtype=dtype)
    host = BinnedDataset.from_dense(X, max_bin=max_bin, zero_as_missing=zam, min_data_in_leaf=1 if n == 1 else 20)
    dev = BinnedDataset.from_dense_device(torch.from_numpy(X).cuda(), max_bin=max_bin, zero_as_missing=zam,
                                          min_data_in_leaf=1 if n == 1 else 20)
    assert dev.on_device and not host.on_device
    assert [f.real for f in dev.features] == [f.real for f in host.features]
    for a, b in zip(dev.features, host.features):
        assert (a.num_bin, a.missing_type, a.default_bin, a.most_freq_bin) == \
               (b.num_bin, b.missing_type, b.default_bin, b.most_freq_bin)
        assert np.array_equal(a.upper_bounds, b.upper_bounds)
    got = dev.bins.cpu().numpy()
    assert np.array_equal(got, host.bins)
    assert np.array_equal(got, _numpy_stored_bins(X, host.features))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_values_on_bounds_and_signed_zero(dtype):
    """Values exactly on an upper bound (or its f32 roundings) go to that bound's bin; -0.0 and
    +0.0 bin alike; +-inf and NaN take the end bins."""
    import torch
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(4)
    X = rng.standard_normal((40000, 3)).astype(dtype)
    X[rng.random(40000) < 0.05, 2] = np.nan
    ds = BinnedDataset.from_dense(X)
    rows = []
    for j, fi in enumerate(ds.features):
        ub = fi.upper_bounds[np.isfinite(fi.upper_bounds)].astype(dtype)
        vals = np.concatenate([ub, np.nextafter(ub, dtype(-np.inf)), np.nextafter(ub, dtype(np.inf)),
                               np.array([0.0, -0.0, np.inf, -np.inf, np.nan], dtype=dtype)])
        block = np.tile(X[:1], (len(vals), 1))
        block[:, fi.real] = vals
        rows.append(block)
    probe = np.concatenate(rows).astype(dtype)
    want = ds.bin_like(probe)
    got = ds.bin_like_device(torch.from_numpy(probe).cuda()).cpu().numpy()
    assert np.array_equal(got, want)
    assert np.array_equal(got, _numpy_stored_bins(probe, ds.features))


def test_learner_from_device_bins_grows_the_same_trees():
    import torch
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig
    X = _values(30000, 20, seed=3, dtype=np.float32)
    host = BinnedDataset.from_dense(X)
    dev = BinnedDataset.from_dense_device(torch.from_numpy(X).cuda())
    rng = np.random.default_rng(0)
    g = rng.standard_normal(len(X)).astype(np.float32)
    h = np.ones(len(X), np.float32)
    for quant in (1, 0):
        c = LearnerConfig(num_leaves=31, use_quantized_grad=quant, stochastic_rounding=1, seed=2,
                          is_constant_hessian=1)
        a, b = GpuTreeLearner(host, c), GpuTreeLearner(dev, c)
        ra, rb = a.train(g, h), b.train(g, h)
        assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])
        assert np.array_equal(a.row_leaf(), b.row_leaf())
        a.close()
        b.close()


def test_device_bins_out_of_range_are_refused():
    """A stored bin past its feature's range is reported by the device check (no compute on it)."""
    import torch
    from lgbm_gb300 import BinnedDataset, LearnerConfig, _lib
    X = _values(5000, 6, seed=8, dtype=np.float64)
    ds = BinnedDataset.from_dense_device(torch.from_numpy(X).cuda())
    bad = ds.bins.clone()
    bad[1, 1234] = 255
    lib = _lib.load()
    feats = ds.feature_array()
    rec = LearnerConfig(num_leaves=7).record()
    h = ctypes.c_void_p()
    rc = lib.bk_learner_create_device_bins(feats.ctypes.data, ds.num_features, bad.data_ptr(), ds.num_data,
                                           rec.ctypes.data, 1, ctypes.byref(h))
    assert rc != 0
    assert "feature 1 row 1234" in _lib.last_error()


def test_bad_bin_mapper_is_refused():
    import torch
    from lgbm_gb300 import BinnedDataset, _lib
    X = _values(1000, 6, seed=9, dtype=np.float64)
    ds = BinnedDataset.from_dense(X)
    lib = _lib.load()
    feats = ds.feature_array()
    offs = np.zeros(ds.num_features + 1, dtype=np.int32)
    for j, fi in enumerate(ds.features):
        offs[j + 1] = offs[j] + fi.num_bin
    offs[-1] += 1  # the last feature's bound count disagrees with its num_bin
    ub = np.zeros(int(offs[-1]), dtype=np.float64)
    Xd = torch.from_numpy(X).cuda()
    out = torch.empty((ds.num_features, len(X)), dtype=torch.uint8, device="cuda")
    rc = lib.bk_bin_dense_device(Xd.data_ptr(), 0, len(X), X.shape[1], feats.ctypes.data, ds.num_features,
                                 ub.ctypes.data, offs.ctypes.data, out.data_ptr(), None)
    assert rc != 0
    assert "bad bin mapper" in _lib.last_error()

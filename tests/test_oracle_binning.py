"""The oracle's own dataset preparation (oracle/binning.cpp) against upstream's bin mappers and
against the product's host binning.

The CPU reference arm of the benchmark bins its rows with the oracle alone, so the oracle's
restatement of the row sample (io/sample.rs:16-19 with utils/random.rs:52-76) and of
BinMapper::find_bin (io/bin.rs:342-554) is pinned here on its own: every numerical feature of the
reference's tests/fixtures/datasets cases must give the BinMapper that upstream's save_binary wrote
(used / trivial, num_bin, missing type, default and most frequent bin, sparse rate, min / max, every
upper bound bit for bit), as crates/lgbm-core/tests/golden_binning.rs:29-63 checks for the reference.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

DATASETS = os.path.join(GOLDEN, "datasets")
CASES = sorted(f[:-5] for f in os.listdir(DATASETS) if f.endswith(".json"))
K_ZERO = float(np.float32(1e-35))


def _oracle_mappers(oracle, X, p, categorical):
    """BinMapper::find_bin of every numerical column over the oracle's LCG row sample."""
    lib = oracle.load()
    n, ncol = X.shape
    k = min(n, int(p.get("bin_construct_sample_cnt", 200000)))
    rows = np.zeros(k, np.int64)
    k = lib.orc_sample_rows(n, k, int(p.get("data_random_seed", 1)), rows.ctypes.data)
    rows = rows[:k]
    filter_cnt = int((float(p.get("min_data_in_leaf", 20)) * k) / float(n))
    max_bins = p.get("max_bin_by_feature") or [int(p.get("max_bin", 255))] * ncol
    out = {}
    for c in range(ncol):
        if c in categorical:
            continue
        vals = np.ascontiguousarray(X[rows, c], dtype=np.float64)
        ub = np.zeros(1024, np.float64)
        meta = np.zeros(4, np.int32)
        dmeta = np.zeros(3, np.float64)
        nb = lib.orc_find_bin(vals.ctypes.data, len(vals), k, int(max_bins[c]), int(p.get("min_data_in_bin", 3)),
                              filter_cnt, int(bool(p.get("feature_pre_filter", True))),
                              int(bool(p.get("use_missing", True))), int(bool(p.get("zero_as_missing", False))),
                              ub.ctypes.data, 1024, meta.ctypes.data, dmeta.ctypes.data)
        assert nb > 0
        out[c] = dict(num_bin=nb, missing_type=int(meta[0]), is_trivial=bool(meta[1]), default_bin=int(meta[2]),
                      most_freq_bin=int(meta[3]), min_val=float(dmeta[0]), max_val=float(dmeta[1]),
                      sparse_rate=float(dmeta[2]), bin_upper_bound=ub[:nb].copy())
    return out


def test_sample_matches_the_lcg_restatement(oracle):
    """The oracle's row sample equals the LCG's Random::sample in both of its branches."""
    from lgbm_gb300.dataset import _Random
    lib = oracle.load()
    for n, k, seed in ((1000, 900, 1), (100000, 2000, 7), (5000, 5000, 3), (10, 1, 2)):
        got = np.zeros(k, np.int64)
        cnt = lib.orc_sample_rows(n, k, seed, got.ctypes.data)
        assert np.array_equal(got[:cnt], _Random(seed).sample(n, k))


@pytest.mark.parametrize("case", CASES)
def test_oracle_bin_mappers_match_upstream(oracle, case):
    P = json.load(open(os.path.join(DATASETS, case + ".json")))
    X = np.load(os.path.join(DATASETS, P["x"]))["x"]
    categorical = set(int(c) for c in P.get("categorical", []))
    ours = _oracle_mappers(oracle, X, P["params"], categorical)
    checked = 0
    for real, m in enumerate(P["mappers"]):
        if real in categorical:
            continue
        where = "%s feature %d" % (case, real)
        o = ours[real]
        used = m is not None and not m["is_trivial"]
        assert (not o["is_trivial"]) == used, where
        if not used:
            continue
        assert m["bin_type"] == 0, where
        for key in ("num_bin", "missing_type", "default_bin", "most_freq_bin", "sparse_rate", "min_val", "max_val"):
            assert o[key] == m[key], "%s: %s" % (where, key)
        assert [float(v).hex() for v in o["bin_upper_bound"]] == [float(v).hex() for v in m["bin_upper_bound"]], where
        checked += 1
    if len(categorical) < X.shape[1]:
        assert checked > 0 or all(m is None or m["is_trivial"] for m in P["mappers"])


def test_oracle_dataset_equals_host_binning(bklib, oracle):
    """Whole datasets binned by the oracle equal the product's host binning, bins and mappers."""
    from lgbm_gb300 import BinnedDataset, synthetic
    for X, _ in (synthetic.l2_steps(n=60000), synthetic.binary_sparse_linear(n=40000, F=30)):
        o = oracle.bin_dense(X, threads=4)
        d = BinnedDataset.from_dense(X, threads=4)
        assert [f.real for f in o.features] == [f.real for f in d.features]
        for a, b in zip(o.features, d.features):
            assert (a.num_bin, a.missing_type, a.default_bin, a.most_freq_bin) == \
                (b.num_bin, b.missing_type, b.default_bin, b.most_freq_bin)
            assert np.array_equal(a.upper_bounds, b.upper_bounds)
        assert np.array_equal(o.bins, d.bins)

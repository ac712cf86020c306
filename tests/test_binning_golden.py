"""The host bin mappers against upstream's own: every case of the reference's
tests/fixtures/datasets (dense, NaN, zero-as-missing, use_missing off, max_bin 2 / 3 / 8 / 15 / 32,
per-feature max_bin, min_data_in_bin 50, no pre-filter, a 5,000-row bin-construction sample,
one-hot and sparse columns, categorical features) is binned by BinnedDataset.from_dense and each
feature's BinMapper is compared field by field with the one upstream's save_binary wrote
(crates/lgbm-core/tests/golden_binning.rs:29-63 runs the same comparison for the reference):
used / trivial features, num_bin, missing type, default and most frequent bin, bin type, sparse
rate, min / max value, and every bin upper bound (bit for bit) or category.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

DATASETS = os.path.join(GOLDEN, "datasets")
CASES = sorted(f[:-5] for f in os.listdir(DATASETS) if f.endswith(".json"))


def _params(P):
    p = P["params"]
    kw = dict(max_bin=int(p.get("max_bin", 255)), min_data_in_bin=int(p.get("min_data_in_bin", 3)),
              min_data_in_leaf=int(p.get("min_data_in_leaf", 20)),
              bin_construct_sample_cnt=int(p.get("bin_construct_sample_cnt", 200000)),
              data_random_seed=int(p.get("data_random_seed", 1)), use_missing=bool(p.get("use_missing", True)),
              zero_as_missing=bool(p.get("zero_as_missing", False)),
              feature_pre_filter=bool(p.get("feature_pre_filter", True)), categorical=P.get("categorical", []))
    if "max_bin_by_feature" in p:
        kw["max_bin_by_feature"] = p["max_bin_by_feature"]
    return kw


def test_cases_present():
    assert len(CASES) == 20


@pytest.mark.parametrize("case", CASES)
def test_bin_mappers_match_upstream(bklib, case):
    from lgbm_gb300 import BinnedDataset
    P = json.load(open(os.path.join(DATASETS, case + ".json")))
    X = np.load(os.path.join(DATASETS, P["x"]))["x"]
    assert X.shape[0] == P["num_data"]
    ds = BinnedDataset.from_dense(X, **_params(P))
    ours = {fi.real: fi for fi in ds.features}
    want = P["mappers"]
    assert len(want) == X.shape[1]
    for real, m in enumerate(want):
        used = m is not None and not m["is_trivial"]
        assert (real in ours) == used, "%s feature %d: used %s" % (case, real, used)
        if not used:
            continue
        fi = ours[real]
        where = "%s feature %d" % (case, real)
        assert fi.num_bin == m["num_bin"], where
        assert fi.missing_type == m["missing_type"], where
        assert fi.default_bin == m["default_bin"], where
        assert fi.most_freq_bin == m["most_freq_bin"], where
        assert fi.bin_type == m["bin_type"], where
        assert fi.sparse_rate == m["sparse_rate"], where
        assert fi.min_val == m["min_val"] and fi.max_val == m["max_val"], where
        if m["bin_type"] == 0:
            assert [float(v).hex() for v in fi.upper_bounds] == [float(v).hex() for v in m["bin_upper_bound"]], where
        else:
            assert [int(v) for v in fi.bin_to_category] == m["bin_2_categorical"], where

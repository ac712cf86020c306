"""The benchmark's per-leaf-size histogram roofline (host arithmetic only, no GPU): which leaf
each histogram launch of a tree builds, and the algorithmic bytes and GB/s of each size class."""
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "bankai-lightgbm_gb300"))


def _splits(pairs):
    from lgbm_gb300 import SPLIT_DTYPE
    s = np.zeros(len(pairs), dtype=SPLIT_DTYPE)
    for i, (lc, rc) in enumerate(pairs):
        s[i]["left_count"] = lc
        s[i]["right_count"] = rc
    return s


def test_launch_rows_follow_the_searched_children():
    import bench
    n = 1000
    # serial.rs:779-825: the smaller child is built unless both children have fewer than
    # 2 * min_data_in_leaf rows; a tree that stopped early leaves its last launches at 0
    rows = bench._hist_launch_rows(_splits([(600, 400), (30, 10), (50, 20)]), n, leaves=6, min_data=20)
    assert rows == [n, 400, 0, 20, 0]
    # a full tree of L leaves has L - 1 launches: the root's, then one per split but the last
    # (whose children are never searched)
    rows = bench._hist_launch_rows(_splits([(700, 300), (200, 100)]), n, leaves=3, min_data=20)
    assert rows == [n, 300]


def test_roofline_by_leaf_size_buckets_and_bytes():
    import bench
    n = 10_000_000
    # 40 features: a 4-bit tile of 32 (16 group bins each) and 8 features of 256 bins
    feats = [SimpleNamespace(group_bins=16)] * 32 + [SimpleNamespace(group_bins=256)] * 8
    ds = SimpleNamespace(features=feats)
    launches = [(n, 1.0), (2_000_000, 0.5), (50_000, 0.01), (50_000, 0.03), (5_000, 0.01)]
    out = bench._roofline_by_leaf_size(launches, ds, n, peak=1000.0)
    assert [b["leaf_rows"] for b in out] == ["root", "1M+", "10k-100k", "<10k"]
    assert [b["launches"] for b in out] == [1, 1, 2, 1]
    bin_bytes = 32 * 0.5 + 8 * 1.0
    slot = (32 * 16 + 8 * 256) * 8.0
    root = out[0]
    assert root["achieved_gbs"] == pytest.approx(round((n * (bin_bytes + 2.0) + slot) / 1e6, 1))
    mid = out[2]
    per = 50_000 * (bin_bytes + 2.0 + 4.0) + slot  # gathered: 4 index bytes a row
    assert mid["mean_us"] == pytest.approx(20.0)
    assert mid["achieved_gbs"] == pytest.approx(round(2 * per / (0.04 * 1e6), 1))
    assert mid["frac"] == pytest.approx(round(mid["achieved_gbs"] / 1000.0, 4), abs=1e-4)

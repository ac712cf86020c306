"""The C-ABI library builds, loads and exports every symbol include/bkgpu.h declares (no GPU
needed); the record layouts the Python mirror uses match the C structs."""
import ctypes
import os
import re

from conftest import ROOT


def test_header_symbols_are_exported(bklib):
    from lgbm_gb300 import _lib
    header = open(os.path.join(ROOT, "include", "bkgpu.h")).read()
    declared = set(re.findall(r"\b(bk_[a-z_]+)\s*\(", header))
    assert declared, "no declarations found"
    missing = [s for s in declared if not hasattr(bklib, s)]
    assert not missing, missing
    assert declared == set(_lib.EXPORTED)


def test_record_layouts():
    from lgbm_gb300 import CONFIG_DTYPE, FEATURE_DTYPE, SPLIT_DTYPE
    assert FEATURE_DTYPE.itemsize == 32
    assert CONFIG_DTYPE.itemsize == 128
    assert SPLIT_DTYPE.itemsize == 152


def test_binning_matches_reference_layout(bklib):
    """Stored bins follow io/dataset.rs:633-685 (most-frequent bin -> 0)."""
    import numpy as np
    from lgbm_gb300 import BinnedDataset
    rng = np.random.default_rng(0)
    X = rng.standard_normal((5000, 3))
    X[:, 1] = np.where(rng.random(5000) < 0.8, 0.0, X[:, 1])  # most frequent bin = the zero bin
    X[rng.random((5000, 3)) < 0.05] = np.nan
    ds = BinnedDataset.from_dense(X)
    for j, fi in enumerate(ds.features):
        assert ds.bins[j].max() < fi.group_bins
    # the zero bin holds exactly the zeros (bin.rs:228-297); for column 1 it is the most frequent
    fi = ds.features[1]
    assert fi.most_freq_bin == fi.default_bin
    assert np.sum(ds.bins[1] == 0) == np.sum(X[:, 1] == 0.0)

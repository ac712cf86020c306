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


def test_invalid_arguments_fail_with_a_message(bklib):
    """The reference c_api's convention (crates/lgbm-capi/src/lib.rs:1-8,78): a failed call returns
    -1 and leaves a message for bk_last_error(). These calls are refused by argument checks that
    run before any CUDA call, so no GPU is needed."""
    import numpy as np
    from lgbm_gb300 import CONFIG_DTYPE, FEATURE_DTYPE, _lib
    P = ctypes.c_void_p
    out = P()
    feats = np.zeros(1, FEATURE_DTYPE)
    cfg = np.zeros(1, CONFIG_DTYPE)
    bins = np.zeros(4, np.uint8)
    cases = [
        (lambda: bklib.bk_learner_create(None, 1, bins.ctypes.data, 4, cfg.ctypes.data, 1, ctypes.byref(out)),
         "invalid arguments"),
        (lambda: bklib.bk_learner_create(feats.ctypes.data, 1, bins.ctypes.data, 4, cfg.ctypes.data, 1,
                                         ctypes.byref(out)), "num_leaves"),
        (lambda: bklib.bk_learner_train(None, None, None, 0, None, 0, None, None, None, None), "invalid arguments"),
        (lambda: bklib.bk_learners_train_batch(None, 0, None, None, 0, 0.0, None, None, None, None, None),
         "invalid arguments"),
        (lambda: bklib.bk_learner_set_feature_mask(None, None), "null learner"),
        (lambda: bklib.bk_learner_set_bynode(None, 0.5, 0, 1), "null learner"),
        (lambda: bklib.bk_learner_autotune(None, None, None, 0, 1, None), "invalid arguments"),
        (lambda: bklib.bk_learner_set_launch_shape(None, None), "invalid arguments"),
        (lambda: bklib.bk_partition_split_noalloc(None, 0, None, 0, None, None, None, None), "invalid arguments"),
        (lambda: bklib.bk_learner_group_create(None, 0, ctypes.byref(out)), "invalid arguments"),
        (lambda: bklib.bk_learner_group_train(None, None, None, 0.0, None, None, None, None, None),
         "invalid arguments"),
        (lambda: bklib.bk_learner_group_autotune(None, None, None, 1, None), "invalid arguments"),
        (lambda: bklib.bk_learner_search_threads(None, None), "invalid arguments"),
        (lambda: bklib.bk_learner_histogram_cache_capacity(None, None), "invalid arguments"),
        (lambda: bklib.bk_learner_reset_histogram_pool_config(None), "null learner"),
        (lambda: bklib.bk_learner_set_objective_weights(None, None, 1.0, 1.0), "invalid arguments"),
    ]
    for call, words in cases:
        assert call() == -1
        assert words in _lib.last_error(), _lib.last_error()


def test_noalloc_partition_refuses_more_rows_than_its_scratch(bklib):
    """The allocation-free partition's fixed scratch holds 1024 row chunks of at most 2^20 rows:
    larger inputs are refused with a message before anything runs on the device."""
    import numpy as np
    from lgbm_gb300 import _lib
    left = ctypes.c_int64()
    route = np.zeros(256, np.uint8)
    rc = bklib.bk_partition_split_noalloc(16, (1 << 30) + 1, 16, 1, route.ctypes.data, 32, ctypes.byref(left),
                                          None)
    assert rc == -1 and "2^30" in _lib.last_error()

"""The allocation-free partition entry point against the learner's own partition.

Some callers of this library cannot allocate device memory (their memory is owned by another
allocator, or an allocation's implicit device synchronization is not acceptable on their path).
`bk_partition_split_noalloc` serves them with a fixed device scratch array. This test drives it
through the C ABI on two calls in a row and checks that each call reproduces the stable partition
that `bk_learner_train` computed for the same split (read back with `bk_learner_row_leaf`).
It is collected last so that a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _split_and_partition(lib, ds, gpu, oracle_lib, g, h, torch):
    from lgbm_gb300.dataset import FEATURE_DTYPE
    splits, leaf_values, root = gpu.train(g, h)
    assert len(splits) == 1, "a two-leaf tree has one split"
    s = splits[0]
    f = int(s["inner_feature"])
    # the route table of the split (data_partition.rs:299-410), from the oracle's restatement
    feat = np.zeros(1, FEATURE_DTYPE)
    fi = ds.features[f]
    feat[0] = (fi.num_bin, fi.missing_type, fi.default_bin, fi.most_freq_bin, fi.penalty, fi.real, 0)
    route = np.zeros(256, np.uint8)
    oracle_lib.orc_route_table(feat.ctypes.data, int(s["threshold"]), int(s["default_left"]), route.ctypes.data)
    n = ds.num_data
    rows_in = torch.arange(n, dtype=torch.int32, device="cuda")
    bins = torch.from_numpy(np.ascontiguousarray(ds.bins[f])).cuda()
    rows_out = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    left = ctypes.c_int64(-1)
    rc = lib.bk_partition_split_noalloc(rows_in.data_ptr(), n, bins.data_ptr(), n, route.ctypes.data,
                                        rows_out.data_ptr(), ctypes.byref(left), None)
    assert rc == 0, lib.bk_last_error()
    got = rows_out.cpu().numpy()
    row_leaf = gpu.row_leaf()
    want_left = np.flatnonzero(row_leaf == 0).astype(np.int32)
    want_right = np.flatnonzero(row_leaf == 1).astype(np.int32)
    assert left.value == len(want_left) == int(s["left_count"])
    assert np.array_equal(got[:left.value], want_left)
    assert np.array_equal(got[left.value:], want_right)


def test_noalloc_partition_matches_learner_partition():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import harness
    from lgbm_gb300 import BinnedDataset, GpuTreeLearner, LearnerConfig, _lib
    lib = _lib.load()
    lib.bk_partition_split_noalloc.restype = ctypes.c_int32
    lib.bk_partition_split_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    rng = np.random.default_rng(3)
    n, F = 50000, 10
    X = rng.standard_normal((n, F))
    X[:, :3] = rng.integers(0, 8, size=(n, 3))
    X[rng.random((n, F)) < 0.1] = np.nan
    ds = BinnedDataset.from_dense(X)
    cfg = LearnerConfig(num_leaves=2, use_quantized_grad=1, stochastic_rounding=0)
    gpu = GpuTreeLearner(ds, cfg)
    orc_lib = harness.load()
    y = np.nan_to_num(X[:, 0]) - np.nan_to_num(X[:, 4]) + rng.normal(0, 0.1, n)
    g = (0.0 - y).astype(np.float32)
    h = np.ones(n, np.float32)
    _split_and_partition(lib, ds, gpu, orc_lib, g, h, torch)
    # a second call in a row, on another split (the scratch keeps the first call's contents)
    g2 = (0.0 - np.nan_to_num(X[:, 2]) * 3.0 + rng.normal(0, 0.1, n)).astype(np.float32)
    _split_and_partition(lib, ds, gpu, orc_lib, g2, h, torch)
    gpu.close()


def _noalloc_lib():
    import ctypes as c
    from lgbm_gb300 import _lib
    lib = _lib.load()
    lib.bk_partition_split_noalloc.restype = c.c_int32
    lib.bk_partition_split_noalloc.argtypes = [c.c_void_p, c.c_int64, c.c_void_p, c.c_int64, c.c_void_p, c.c_void_p,
                                               c.c_void_p, c.c_void_p]
    return lib


def test_noalloc_partition_many_tiles_per_block_and_gathered_rows():
    """More rows than 1024 blocks of one 2048-row tile: every block walks several tiles, carrying its
    running left count from tile to tile. The input is a permuted subset of the rows (a gathered,
    non-identity row list), checked against a numpy stable partition on two calls in a row."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _noalloc_lib()
    rng = np.random.default_rng(11)
    bins_len = 3_000_000
    bins_np = rng.integers(0, 256, size=bins_len, dtype=np.uint8)
    bins = torch.from_numpy(bins_np).cuda()
    for rows_cnt, seed in ((2_500_000, 1), (2_300_001, 2)):
        r = np.random.default_rng(seed)
        rows_np = r.permutation(bins_len)[:rows_cnt].astype(np.int32)
        route = (r.random(256) < 0.4).astype(np.uint8)
        rows_in = torch.from_numpy(rows_np).cuda()
        rows_out = torch.full((rows_cnt,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        left = ctypes.c_int64(-1)
        rc = lib.bk_partition_split_noalloc(rows_in.data_ptr(), rows_cnt, bins.data_ptr(), bins_len,
                                            route.ctypes.data, rows_out.data_ptr(), ctypes.byref(left), None)
        assert rc == 0, lib.bk_last_error()
        goes_left = route[bins_np[rows_np]] != 0
        want = np.concatenate([rows_np[goes_left], rows_np[~goes_left]])
        assert left.value == int(goes_left.sum())
        assert np.array_equal(rows_out.cpu().numpy(), want)


def test_noalloc_partition_rejects_rows_outside_the_bins_column():
    """A row id at or past bins_len is never read; the call fails with -1 and a message, and the next
    call (whose error flag starts at zero again) succeeds."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _noalloc_lib()
    bins_len = 5000
    bins = torch.zeros(bins_len, dtype=torch.uint8, device="cuda")
    route = np.ones(256, np.uint8)
    rows_bad = torch.tensor([0, 1, bins_len, 3], dtype=torch.int32, device="cuda")
    out = torch.empty(4, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    left = ctypes.c_int64(-1)
    rc = lib.bk_partition_split_noalloc(rows_bad.data_ptr(), 4, bins.data_ptr(), bins_len, route.ctypes.data,
                                        out.data_ptr(), ctypes.byref(left), None)
    assert rc == -1
    assert b"outside the bins column" in lib.bk_last_error()
    rows_ok = torch.tensor([4, 2, 0], dtype=torch.int32, device="cuda")
    rc = lib.bk_partition_split_noalloc(rows_ok.data_ptr(), 3, bins.data_ptr(), bins_len, route.ctypes.data,
                                        out.data_ptr(), ctypes.byref(left), None)
    assert rc == 0, lib.bk_last_error()
    assert left.value == 3 and out[:3].cpu().tolist() == [4, 2, 0]

"""Host-side dataset construction for the GB300 learner.

The learner consumes a binned dataset: one stored-bin column per inner feature plus each
feature's bin-mapper facts (num_bin, missing type, default bin, most frequent bin). In
bankai-lightgbm the host builds this with ``Dataset::from_dense`` (crates/lgbm-core/src/io/
dataset.rs:904-983) and keeps the bin mappers; this module does the same for dense numerical
data so the learner can be driven without the Rust host:

* row sample for bin construction — ``create_sample_indices`` (io/sample.rs:11-14) with the
  LCG ``Random::sample`` (utils/random.rs:52-76);
* one ``BinMapper::find_bin`` per column (io/bin.rs:342-554), done in C++ by
  ``bk_find_bin_numerical``;
* trivial features dropped (io/dataset.rs:389-393); every used feature is its own dense group
  (dense data never bundles: io/dataset.rs:171-177), stored bins written by
  ``bk_values_to_group_bins`` (io/dataset.rs:633-685).

Numerical and categorical features (``categorical=`` column list) are supported.
"""
from concurrent.futures import ThreadPoolExecutor
import math

import numpy as np

from . import _lib

K_ZERO_THRESHOLD = float(np.float32(1e-35))
MISSING_NONE, MISSING_ZERO, MISSING_NAN = 0, 1, 2
BIN_NUMERICAL, BIN_CATEGORICAL = 0, 1


class _Random:
    """utils/random.rs:7-76 — the MSVC-style LCG used by LightGBM's sampling."""

    def __init__(self, seed: int):
        self.x = seed & 0xFFFFFFFF

    def _int16(self):
        self.x = (self.x * 214013 + 2531011) & 0xFFFFFFFF
        return (self.x >> 16) & 0x7FFF

    def _int32(self):
        self.x = (self.x * 214013 + 2531011) & 0xFFFFFFFF
        return self.x & 0x7FFFFFFF

    def next_int(self, lower, upper):
        return self._int32() % (upper - lower) + lower

    def next_float(self):
        return np.float32(self._int16()) / np.float32(32768.0)

    def sample(self, n, k):
        if k > n or k <= 0:
            return np.zeros(0, dtype=np.int64)
        if k == n:
            return np.arange(n, dtype=np.int64)
        if k > 1 and float(k) > float(n) / math.log2(k):
            ret = []
            for i in range(n):
                prob = (k - len(ret)) / float(n - i)
                if float(self.next_float()) < prob:
                    ret.append(i)
            return np.asarray(ret, dtype=np.int64)
        s = set()
        for r in range(n - k, n):
            v = self.next_int(0, r + 1)
            if v in s:
                s.add(r)
            else:
                s.add(v)
        return np.asarray(sorted(s), dtype=np.int64)


class FeatureInfo:
    __slots__ = ("real", "num_bin", "missing_type", "default_bin", "most_freq_bin", "upper_bounds", "penalty",
                 "min_val", "max_val", "sparse_rate", "bin_type", "bin_to_category")

    def __init__(self):
        self.bin_type = BIN_NUMERICAL
        self.bin_to_category = None

    @property
    def offset(self):
        return 1 if self.most_freq_bin == 0 else 0

    @property
    def group_bins(self):
        """Stored bins of the feature's group: bin 0 holds the most-frequent-bin rows."""
        return 1 + self.num_bin - self.offset

    @property
    def categorical(self):
        return self.bin_type == BIN_CATEGORICAL

    def bin_to_value(self, b):
        """BinMapper::bin_to_value (io/bin.rs:593-599): the bound of a numerical bin, the category
        code of a categorical one."""
        if self.categorical:
            return float(self.bin_to_category[b])
        return float(self.upper_bounds[b])


class BinnedDataset:
    """A dense dataset in the learner's input form.

    ``bins``: uint8 array ``[num_features, num_data]`` of stored group bins (column-major).
    ``features``: per inner feature, its ``FeatureInfo``.
    """

    def __init__(self, bins, features, num_total_features):
        self.bins = bins
        self.features = features
        self.num_total_features = num_total_features

    @property
    def on_device(self):
        """True when ``bins`` is a CUDA tensor (``from_dense_device``)."""
        return bool(getattr(self.bins, "is_cuda", False))

    @property
    def num_data(self):
        return self.bins.shape[1]

    @property
    def num_features(self):
        return len(self.features)

    @classmethod
    def from_dense(cls, X, max_bin=255, min_data_in_bin=3, min_data_in_leaf=20, bin_construct_sample_cnt=200000,
                   data_random_seed=1, use_missing=True, zero_as_missing=False, feature_pre_filter=True,
                   threads=8, categorical=(), max_bin_by_feature=None):
        """``categorical``: the column indices binned as categories (io/dataset.rs from_dense's
        categorical list); the others are numerical. ``max_bin_by_feature``: one max_bin per
        column (io/sample.rs:136-175), or None for ``max_bin`` everywhere."""
        X = np.asarray(X)
        n, ncol = X.shape
        if max_bin_by_feature is not None:
            max_bin = [int(b) for b in max_bin_by_feature]
            if len(max_bin) != ncol or min(max_bin) <= 1:
                raise ValueError("max_bin_by_feature needs one value > 1 per column")
        if max(max_bin if isinstance(max_bin, list) else [max_bin]) > 255:
            raise ValueError("max_bin above 255 needs 16-bit stored bins, which this learner does not take")
        rows = _Random(data_random_seed).sample(n, min(n, bin_construct_sample_cnt))
        features = _find_mappers(lambda col: np.asarray(X[rows, col], dtype=np.float64), ncol, n, len(rows),
                                 max_bin, min_data_in_bin, min_data_in_leaf, use_missing, zero_as_missing,
                                 feature_pre_filter, threads, categorical)
        ds = cls(None, features, ncol)
        ds.bins = ds.bin_like(X, threads=threads)
        return ds

    def bin_like(self, X, threads=8):
        """Stored bins of new rows with this dataset's bin mappers (held-out / validation data,
        io/dataset.rs:987-1003 from_dense_reference)."""
        X = np.asarray(X)
        lib = _lib.load()
        n = X.shape[0]
        bins = np.zeros((self.num_features, n), dtype=np.uint8)

        def fill(j):
            fi = self.features[j]
            col = np.ascontiguousarray(X[:, fi.real], dtype=np.float64)
            if fi.categorical:
                lib.bk_values_to_group_bins_categorical(col.ctypes.data, n, 1, fi.bin_to_category.ctypes.data,
                                                        fi.num_bin, fi.most_freq_bin, bins[j].ctypes.data)
            else:
                lib.bk_values_to_group_bins(col.ctypes.data, n, 1, fi.upper_bounds.ctypes.data, fi.num_bin,
                                            fi.missing_type, fi.most_freq_bin, bins[j].ctypes.data)

        with ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(fill, range(self.num_features)))
        return bins

    @classmethod
    def from_dense_device(cls, X, max_bin=255, min_data_in_bin=3, min_data_in_leaf=20, bin_construct_sample_cnt=200000,
                          data_random_seed=1, use_missing=True, zero_as_missing=False, feature_pre_filter=True,
                          threads=8):
        """As ``from_dense`` for a row-major CUDA tensor ``X`` ([num_data, num_columns], float32 or
        float64): the bin mappers come from the same row sample (copied to the host), the stored
        bins are written on the device by ``bk_bin_dense_device``; ``bins`` is a uint8 CUDA tensor
        [num_features, num_data]."""
        import torch
        if max_bin > 255:
            raise ValueError("max_bin above 255 needs 16-bit stored bins, which this learner does not take")
        if not (X.is_cuda and X.dim() == 2 and X.dtype in (torch.float32, torch.float64)):
            raise ValueError("X must be a 2-D float32 / float64 CUDA tensor")
        X = X.contiguous()
        n, ncol = X.shape
        rows = _Random(data_random_seed).sample(n, min(n, bin_construct_sample_cnt))
        sample = X[torch.as_tensor(rows, device=X.device)].double().cpu().numpy()
        features = _find_mappers(lambda col: sample[:, col], ncol, n, len(rows), max_bin, min_data_in_bin,
                                 min_data_in_leaf, use_missing, zero_as_missing, feature_pre_filter, threads, ())
        ds = cls(None, features, ncol)
        ds.bins = ds.bin_like_device(X)
        return ds

    def bin_like_device(self, X):
        """Stored bins of the rows of a row-major CUDA tensor ``X`` with this dataset's bin mappers,
        on the device (uint8 CUDA tensor [num_features, rows])."""
        import torch
        X = X.contiguous()
        n, ncol = X.shape
        if any(fi.categorical for fi in self.features):
            raise ValueError("device binning takes numerical features only; bin categorical data with bin_like")
        out = torch.empty((len(self.features), n), dtype=torch.uint8, device=X.device)
        if not self.features:
            return out
        lib = _lib.load()
        feats = self.feature_array()
        offs = np.zeros(len(self.features) + 1, dtype=np.int32)
        for j, fi in enumerate(self.features):
            offs[j + 1] = offs[j] + fi.num_bin
        ub = np.concatenate([fi.upper_bounds for fi in self.features]).astype(np.float64)
        vt = 0 if X.dtype == torch.float64 else 1
        stream = torch.cuda.current_stream(X.device).cuda_stream
        _lib.check(lib.bk_bin_dense_device(X.data_ptr(), vt, n, ncol, feats.ctypes.data, len(self.features),
                                           ub.ctypes.data, offs.ctypes.data, out.data_ptr(), stream),
                   "bk_bin_dense_device")
        return out

    def feature_array(self):
        """The ``bk_feature`` records of include/bkgpu.h, as a numpy structured array."""
        arr = np.zeros(self.num_features, dtype=FEATURE_DTYPE)
        for j, fi in enumerate(self.features):
            arr[j] = (fi.num_bin, fi.missing_type, fi.default_bin, fi.most_freq_bin, fi.penalty, fi.real, fi.bin_type)
        return arr


def _find_mappers(sample_col, ncol, n, sample_cnt, max_bin, min_data_in_bin, min_data_in_leaf, use_missing,
                  zero_as_missing, feature_pre_filter, threads, categorical=()):
    """``BinMapper::find_bin`` (io/bin.rs:342-554) for every column over the sampled rows
    (``sample_col(col)``: the column's sampled values, f64), categorical for the columns in
    ``categorical``, dropping trivial features (io/dataset.rs:389-393)."""
    lib = _lib.load()
    filter_cnt = int((float(min_data_in_leaf) * sample_cnt) / float(n))
    cap = 1024
    cat_cols = set(int(c) for c in categorical)
    max_bins = max_bin if isinstance(max_bin, list) else [max_bin] * ncol

    def find(col):
        max_bin = max_bins[col]
        vals = np.asarray(sample_col(col), dtype=np.float64)
        keep = (np.abs(vals) > K_ZERO_THRESHOLD) | np.isnan(vals)
        vals = np.ascontiguousarray(vals[keep])
        meta = np.zeros(4, dtype=np.int32)
        dmeta = np.zeros(3, dtype=np.float64)
        fi = FeatureInfo()
        if col in cat_cols:
            b2c = np.zeros(cap, dtype=np.int32)
            nb = lib.bk_find_bin_categorical(vals.ctypes.data, len(vals), sample_cnt, max_bin, min_data_in_bin,
                                             filter_cnt, int(feature_pre_filter), int(use_missing),
                                             int(zero_as_missing), b2c.ctypes.data, cap, meta.ctypes.data,
                                             dmeta.ctypes.data)
            if nb < 0:
                raise RuntimeError("bin mapper capacity exceeded")
            fi.bin_type = BIN_CATEGORICAL
            fi.bin_to_category = b2c[:nb].copy()
            ub = np.zeros(0)
        else:
            ub = np.zeros(cap, dtype=np.float64)
            nb = lib.bk_find_bin_numerical(vals.ctypes.data, len(vals), sample_cnt, max_bin, min_data_in_bin,
                                           filter_cnt, int(feature_pre_filter), int(use_missing),
                                           int(zero_as_missing), ub.ctypes.data, cap, meta.ctypes.data,
                                           dmeta.ctypes.data)
            if nb < 0:
                raise RuntimeError("bin mapper capacity exceeded")
        fi.real = col
        fi.num_bin = int(nb)
        fi.missing_type = int(meta[0])
        fi.default_bin = int(meta[2])
        fi.most_freq_bin = int(meta[3])
        fi.upper_bounds = ub[:nb].copy()
        fi.penalty = 1.0
        fi.min_val, fi.max_val, fi.sparse_rate = float(dmeta[0]), float(dmeta[1]), float(dmeta[2])
        return fi, bool(meta[1])

    with ThreadPoolExecutor(max_workers=threads) as ex:
        found = list(ex.map(find, range(ncol)))
    return [fi for fi, trivial in found if not trivial]


FEATURE_DTYPE = np.dtype([("num_bin", np.int32), ("missing_type", np.int32), ("default_bin", np.int32),
                          ("most_freq_bin", np.int32), ("penalty", np.float64), ("real_feature", np.int32),
                          ("bin_type", np.int32)], align=True)

"""The oracle's histogram construction against the reference's own histogram checks (no GPU):

* integer histograms of packed int8 gradient / uint8 hessian values against the brute-force
  per-bin sums of crates/lgbm-core/tests/quantized_int_histogram.rs:15-104 (its vectors and its
  overflow-of-the-narrower-width cases);
* float histograms against the ordered f64 sums of crates/lgbm-core/tests/simd_histogram.rs:7-54:
  repeated destinations, a descending row subset, and a gradient pattern of cancelling and
  disparate magnitudes (1e20, 1, -1e20, -0.0, the smallest normal f32, -3.25, 0.5) that exposes
  any change of addition order — compared bit for bit.
"""
import numpy as np
import pytest


def _pack(g, h):
    """(int8 gradient << 8) | uint8 hessian as an int16 (int_histogram.rs:38-40)."""
    return np.array([((g & 0xFF) << 8) | (h & 0xFF)], dtype=np.int32).astype(np.uint16).astype(np.int16)[0]


def _int_hist(oracle, bins_col, packed, group_bins, rows=None):
    lib = oracle.load()
    n = len(bins_col)
    col = np.ascontiguousarray(bins_col, dtype=np.uint8)
    gb = np.array([group_bins], dtype=np.int32)
    pk = np.ascontiguousarray(packed, dtype=np.int16)
    out_g = np.zeros(group_bins, np.int64)
    out_h = np.zeros(group_bins, np.int64)
    r = None if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
    lib.orc_hist_int(col.ctypes.data, n, 1, gb.ctypes.data, None if r is None else r.ctypes.data,
                     n if r is None else len(r), pk.ctypes.data, out_g.ctypes.data, out_h.ctypes.data)
    return out_g, out_h


def _brute(packed, bins, num_bins):
    g = np.zeros(num_bins, np.int64)
    h = np.zeros(num_bins, np.int64)
    for p, b in zip(packed, bins):
        g[b] += int(np.int8(np.int16(p) >> 8))
        h[b] += int(np.uint16(np.int16(p)) & 0xFF)
    return g, h


def test_int_histogram_matches_bruteforce(oracle):
    pairs = [(3, 2), (-5, 4), (1, 1), (-2, 7), (6, 3), (-1, 2), (0, 5), (4, 1)]
    packed = np.array([_pack(g, h) for g, h in pairs], dtype=np.int16)
    bins = np.array([0, 1, 0, 2, 1, 2, 0, 1], dtype=np.uint8)
    got = _int_hist(oracle, bins, packed, 3)
    want = _brute(packed, bins, 3)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("rows,g,h,want", [(500, 50, 50, (25000, 25000)), (70000, 100, 200, (7000000, 14000000))])
def test_int_histogram_holds_sums_beyond_narrow_widths(oracle, rows, g, h, want):
    packed = np.full(rows, _pack(g, h), dtype=np.int16)
    bins = np.zeros(rows, dtype=np.uint8)
    og, oh = _int_hist(oracle, bins, packed, 1)
    assert (int(og[0]), int(oh[0])) == want


@pytest.mark.parametrize("num_bin", [16, 255])
@pytest.mark.parametrize("n", [0, 1, 3, 17, 257])
@pytest.mark.parametrize("subset", [False, True])
@pytest.mark.parametrize("constant", [False, True])
def test_float_histogram_is_the_ordered_sum(oracle, num_bin, n, subset, constant):
    lib = oracle.load()
    bins = np.array([(r // 7) % 3 for r in range(n)], dtype=np.uint8)
    rows = np.arange(n - 1, -1, -2, dtype=np.int32)  # descending, every other row
    indices = rows if subset else np.arange(n, dtype=np.int32)
    pattern = np.array([1e20, 1.0, -1e20, -0.0, np.finfo(np.float32).tiny, -3.25, 0.5], dtype=np.float32)
    g = np.array([pattern[r % 7] for r in range(n)], dtype=np.float32)
    h = np.array([(r % 11) * 0.125 for r in range(n)], dtype=np.float32)
    if constant and n:
        h[:] = 1.0  # a constant hessian: the slot counts rows, scaled by hessians[0]
    want = np.zeros(2 * num_bin, dtype=np.float64)
    for r in indices:
        want[2 * bins[r]] += float(g[r])
        want[2 * bins[r] + 1] += 1.0 if constant else float(h[r])
    got = np.zeros(2 * num_bin, dtype=np.float64)
    gb = np.array([num_bin], dtype=np.int32)
    col = np.ascontiguousarray(bins)
    lib.orc_hist_float(col.ctypes.data, n, 1, gb.ctypes.data, rows.ctypes.data if subset else None,
                       len(indices), g.ctypes.data, h.ctypes.data, int(constant), got.ctypes.data)
    assert [x.hex() for x in got.tolist()] == [x.hex() for x in want.tolist()]

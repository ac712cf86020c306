// Host-side dataset preparation: numerical bin mappers.
//
// The GB300 learner consumes already-binned feature columns, exactly like bankai-lightgbm's
// SerialTreeLearner consumes a Dataset whose BinMappers the host keeps. This file restates the
// numerical part of `BinMapper::find_bin` (crates/lgbm-core/src/io/bin.rs:342-554) so that a
// caller without the Rust host (the Python harness, the benchmark) can build the same bins.
// Categorical bin mappers (the categorical branch of find_bin) are restated too; forced bin bounds
// are not supported here.
//
// Compiled with -ffp-contract=off: the bound arithmetic must round exactly as the reference.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

const double K_ZERO_THRESHOLD = (double)1e-35f;  // meta.rs:4
const double K_SPARSE_THRESHOLD = 0.7;           // bin.rs:9

inline double next_up(double a) { return std::nextafter(a, INFINITY); }
inline bool check_double_equal_ordered(double a, double b) { return b <= next_up(a); }

// bin.rs:51-137 — GreedyFindBin.
std::vector<double> greedy_find_bin(const double* dv, const int32_t* counts, size_t ndv, int32_t max_bin,
                                    size_t total_cnt, int32_t min_data_in_bin) {
  std::vector<double> ub;
  if ((int64_t)ndv <= (int64_t)max_bin) {
    int32_t cur = 0;
    for (size_t i = 0; i + 1 < ndv; ++i) {
      cur += counts[i];
      if (cur >= min_data_in_bin) {
        double val = next_up((dv[i] + dv[i + 1]) / 2.0);
        if (ub.empty() || !check_double_equal_ordered(ub.back(), val)) {
          ub.push_back(val);
          cur = 0;
        }
      }
    }
    ub.push_back(INFINITY);
    return ub;
  }
  if (min_data_in_bin > 0) {
    max_bin = std::min(max_bin, (int32_t)(total_cnt / (size_t)min_data_in_bin));
    max_bin = std::max(max_bin, 1);
  }
  double mean_bin_size = (double)total_cnt / (double)max_bin;
  int32_t rest_bin_cnt = max_bin;
  int32_t rest_sample_cnt = (int32_t)total_cnt;
  std::vector<uint8_t> big(ndv, 0);
  for (size_t i = 0; i < ndv; ++i) {
    if ((double)counts[i] >= mean_bin_size) {
      big[i] = 1;
      rest_bin_cnt -= 1;
      rest_sample_cnt -= counts[i];
    }
  }
  mean_bin_size = (double)rest_sample_cnt / (double)rest_bin_cnt;
  std::vector<double> upper((size_t)max_bin, INFINITY), lower((size_t)max_bin, INFINITY);
  size_t bin_cnt = 0;
  lower[0] = dv[0];
  int32_t cur = 0;
  for (size_t i = 0; i + 1 < ndv; ++i) {
    if (!big[i]) rest_sample_cnt -= counts[i];
    cur += counts[i];
    double half = mean_bin_size * 0.5;
    if (big[i] || (double)cur >= mean_bin_size || (big[i + 1] && (double)cur >= std::max(1.0, half))) {
      upper[bin_cnt] = dv[i];
      bin_cnt += 1;
      lower[bin_cnt] = dv[i + 1];
      if ((int32_t)bin_cnt >= max_bin - 1) break;
      cur = 0;
      if (!big[i]) {
        rest_bin_cnt -= 1;
        mean_bin_size = (double)rest_sample_cnt / (double)rest_bin_cnt;
      }
    }
  }
  bin_cnt += 1;
  for (size_t i = 0; i + 1 < bin_cnt; ++i) {
    double val = next_up((upper[i] + lower[i + 1]) / 2.0);
    if (ub.empty() || !check_double_equal_ordered(ub.back(), val)) ub.push_back(val);
  }
  ub.push_back(INFINITY);
  return ub;
}

// bin.rs:228-297 — FindBinWithZeroAsOneBin (no forced bounds).
std::vector<double> find_bin_zero_as_one(const std::vector<double>& dv, const std::vector<int32_t>& counts,
                                         int32_t max_bin, size_t total_sample_cnt, int32_t min_data_in_bin) {
  size_t n = dv.size();
  std::vector<double> ub;
  int32_t left_cnt_data = 0, cnt_zero = 0, right_cnt_data = 0;
  for (size_t i = 0; i < n; ++i) {
    if (dv[i] <= -K_ZERO_THRESHOLD) left_cnt_data += counts[i];
    else if (dv[i] > K_ZERO_THRESHOLD) right_cnt_data += counts[i];
    else cnt_zero += counts[i];
  }
  size_t left_cnt = n;
  for (size_t i = 0; i < n; ++i)
    if (dv[i] > -K_ZERO_THRESHOLD) {
      left_cnt = i;
      break;
    }
  if (left_cnt > 0 && max_bin > 1) {
    double denom = (double)total_sample_cnt - (double)cnt_zero;
    int32_t left_max_bin = (int32_t)((double)left_cnt_data / denom * (double)(max_bin - 1));
    left_max_bin = std::max(left_max_bin, 1);
    ub = greedy_find_bin(dv.data(), counts.data(), left_cnt, left_max_bin, (size_t)left_cnt_data, min_data_in_bin);
    if (!ub.empty()) ub.back() = -K_ZERO_THRESHOLD;
  }
  long right_start = -1;
  for (size_t i = left_cnt; i < n; ++i)
    if (dv[i] > K_ZERO_THRESHOLD) {
      right_start = (long)i;
      break;
    }
  int32_t right_max_bin = max_bin - 1 - (int32_t)ub.size();
  if (right_start >= 0 && right_max_bin > 0) {
    std::vector<double> right = greedy_find_bin(dv.data() + right_start, counts.data() + right_start,
                                                n - (size_t)right_start, right_max_bin, (size_t)right_cnt_data,
                                                min_data_in_bin);
    ub.push_back(K_ZERO_THRESHOLD);
    ub.insert(ub.end(), right.begin(), right.end());
  } else {
    ub.push_back(INFINITY);
  }
  return ub;
}

// bin.rs:300-319 — NeedFilter (numerical).
bool need_filter(const std::vector<int32_t>& cnt_in_bin, int32_t total_cnt, int32_t filter_cnt) {
  int32_t sum_left = 0;
  for (size_t i = 0; i + 1 < cnt_in_bin.size(); ++i) {
    sum_left += cnt_in_bin[i];
    if (sum_left >= filter_cnt && total_cnt - sum_left >= filter_cnt) return false;
  }
  return true;
}

// The preamble of BinMapper::find_bin (bin.rs:342-406) shared by both bin types: NaN values
// compacted out (the missing type follows use_missing / zero_as_missing / whether NaNs occur), the
// rest sorted, and the distinct values with their counts, zeros (implied by total_sample_cnt)
// inserted where they sort.
void distinct_sample(double* values, int64_t num_values, int64_t total_sample_cnt, int32_t use_missing,
                     int32_t zero_as_missing, int32_t* missing_out, size_t* na_out, std::vector<double>* dv_out,
                     std::vector<int32_t>* counts_out) {
  size_t nsv = (size_t)num_values;
  size_t non_na = 0;
  for (size_t i = 0; i < nsv; ++i)
    if (!std::isnan(values[i])) values[non_na++] = values[i];
  size_t na_cnt = 0;
  int32_t missing;
  if (!use_missing) missing = 0;
  else if (zero_as_missing) missing = 1;
  else if (non_na == nsv) missing = 0;
  else {
    na_cnt = nsv - non_na;
    missing = 2;
  }
  nsv = non_na;
  int32_t zero_cnt = (int32_t)((size_t)total_sample_cnt - nsv - na_cnt);
  std::stable_sort(values, values + nsv, [](double a, double b) { return a < b; });
  std::vector<double>& dv = *dv_out;
  std::vector<int32_t>& counts = *counts_out;
  if (nsv == 0 || (values[0] > 0.0 && zero_cnt > 0)) {
    dv.push_back(0.0);
    counts.push_back(zero_cnt);
  }
  if (nsv > 0) {
    dv.push_back(values[0]);
    counts.push_back(1);
  }
  for (size_t i = 1; i < nsv; ++i) {
    if (!check_double_equal_ordered(values[i - 1], values[i])) {
      if (values[i - 1] < 0.0 && values[i] > 0.0) {
        dv.push_back(0.0);
        counts.push_back(zero_cnt);
      }
      dv.push_back(values[i]);
      counts.push_back(1);
    } else {
      dv.back() = values[i];
      counts.back() += 1;
    }
  }
  if (nsv > 0 && values[nsv - 1] < 0.0 && zero_cnt > 0) {
    dv.push_back(0.0);
    counts.push_back(zero_cnt);
  }
  *missing_out = missing;
  *na_out = na_cnt;
}

// Rust's saturating `f64 as i32` (NaN -> 0): the categorical code of a value.
int32_t cat_code(double v) {
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0) return INT32_MAX;
  if (v <= -2147483648.0) return INT32_MIN;
  return (int32_t)v;  // truncation toward zero
}

}  // namespace

extern "C" {

// One numerical BinMapper (bin.rs:342-554). `values` holds the sampled values whose magnitude is
// above kZeroThreshold or that are NaN (zeros are implied by `total_sample_cnt`); it is modified in
// place (compacted and sorted, as the reference does). Writes up to `cap` upper bounds and
// returns num_bin, or -1 when `cap` is too small. meta_out = {missing_type, is_trivial,
// default_bin, most_freq_bin}; dmeta_out = {min_val, max_val, sparse_rate}.
int32_t bk_find_bin_numerical(double* values, int64_t num_values, int64_t total_sample_cnt, int32_t max_bin,
                              int32_t min_data_in_bin, int32_t min_split_data, int32_t pre_filter,
                              int32_t use_missing, int32_t zero_as_missing, double* upper_bounds, int32_t cap,
                              int32_t* meta_out, double* dmeta_out) {
  int32_t missing = 0;
  size_t na_cnt = 0;
  std::vector<double> dv;
  std::vector<int32_t> counts;
  distinct_sample(values, num_values, total_sample_cnt, use_missing, zero_as_missing, &missing, &na_cnt, &dv,
                  &counts);
  double min_val = dv.front(), max_val = dv.back();
  std::vector<double> ub;
  if (missing == 1) {
    ub = find_bin_zero_as_one(dv, counts, max_bin, (size_t)total_sample_cnt, min_data_in_bin);
    if (ub.size() == 2) missing = 0;
  } else if (missing == 0) {
    ub = find_bin_zero_as_one(dv, counts, max_bin, (size_t)total_sample_cnt, min_data_in_bin);
  } else {
    ub = find_bin_zero_as_one(dv, counts, max_bin - 1, (size_t)total_sample_cnt - na_cnt, min_data_in_bin);
    ub.push_back(2.0);  // bin.rs:441-444: the stored bound of the NaN bin is MissingType::NaN as f64
  }
  int32_t num_bin = (int32_t)ub.size();
  std::vector<int32_t> cnt_in_bin((size_t)num_bin, 0);
  size_t i_bin = 0;
  for (size_t i = 0; i < dv.size(); ++i) {
    while (dv[i] > ub[i_bin] && (int32_t)i_bin < num_bin - 1) ++i_bin;
    cnt_in_bin[i_bin] += counts[i];
  }
  if (missing == 2) cnt_in_bin.back() = (int32_t)na_cnt;
  bool is_trivial = num_bin <= 1;
  if (!is_trivial && pre_filter && need_filter(cnt_in_bin, (int32_t)total_sample_cnt, min_split_data))
    is_trivial = true;
  int32_t default_bin = 0, mfb = 0;
  double sparse_rate = 1.0;
  if (!is_trivial) {
    // value_to_bin(0.0) (bin.rs:558-589)
    int32_t l = 0, r = num_bin - 1;
    if (missing == 2) r -= 1;
    while (l < r) {
      int32_t mid = (r + l - 1) / 2;
      if (0.0 <= ub[(size_t)mid]) r = mid;
      else l = mid + 1;
    }
    default_bin = l;
    size_t am = 0;
    for (size_t i = 1; i < cnt_in_bin.size(); ++i)
      if (cnt_in_bin[i] > cnt_in_bin[am]) am = i;
    mfb = (int32_t)am;
    double max_sparse_rate = (double)cnt_in_bin[(size_t)mfb] / (double)total_sample_cnt;
    if (mfb != default_bin && max_sparse_rate < K_SPARSE_THRESHOLD) mfb = default_bin;
    sparse_rate = (double)cnt_in_bin[(size_t)mfb] / (double)total_sample_cnt;
  }
  if (num_bin > cap) return -1;
  for (int32_t i = 0; i < num_bin; ++i) upper_bounds[i] = ub[(size_t)i];
  meta_out[0] = missing;
  meta_out[1] = is_trivial ? 1 : 0;
  meta_out[2] = default_bin;
  meta_out[3] = mfb;
  dmeta_out[0] = min_val;
  dmeta_out[1] = max_val;
  dmeta_out[2] = sparse_rate;
  return num_bin;
}

// One categorical BinMapper (bin.rs:459-554, the categorical branch of find_bin): the sampled
// values truncated to integer codes (negative codes count as missing), the codes sorted by count
// (descending, stable), bin 0 for "other / missing" and one bin per code until 99% of the
// non-missing sample is covered or max_bin codes are used (codes rarer than min_data_in_bin end it
// after the second). `values` as for bk_find_bin_numerical (modified in place). Writes up to `cap`
// codes of the bins (bin_to_category[0] = -1) and returns num_bin, or -1 when `cap` is too small.
// meta_out = {missing_type, is_trivial, default_bin, most_freq_bin}; dmeta_out = {min_val,
// max_val, sparse_rate}.
int32_t bk_find_bin_categorical(double* values, int64_t num_values, int64_t total_sample_cnt, int32_t max_bin,
                                int32_t min_data_in_bin, int32_t min_split_data, int32_t pre_filter,
                                int32_t use_missing, int32_t zero_as_missing, int32_t* bin_to_category, int32_t cap,
                                int32_t* meta_out, double* dmeta_out) {
  int32_t missing = 0;
  size_t na_cnt = 0;
  std::vector<double> dv;
  std::vector<int32_t> counts;
  distinct_sample(values, num_values, total_sample_cnt, use_missing, zero_as_missing, &missing, &na_cnt, &dv,
                  &counts);
  double min_val = dv.front(), max_val = dv.back();
  std::vector<int32_t> codes, code_counts;
  for (size_t i = 0; i < dv.size(); ++i) {
    const int32_t val = cat_code(dv[i]);
    if (val < 0) {
      na_cnt += (size_t)counts[i];
    } else if (codes.empty() || codes.back() != val) {
      codes.push_back(val);
      code_counts.push_back(counts[i]);
    } else {
      code_counts.back() += counts[i];
    }
  }
  std::vector<int32_t> b2c;
  std::vector<int32_t> cnt_in_bin;
  int32_t num_bin = 1;  // BinMapper::default(): one bin
  const int64_t rest_cnt = total_sample_cnt - (int64_t)na_cnt;
  if (rest_cnt > 0) {
    // SortForPair(counts, values, 0, reverse): stable, by count descending
    std::vector<size_t> order(codes.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return code_counts[a] > code_counts[b]; });
    std::vector<int32_t> sc(order.size()), scnt(order.size());
    for (size_t i = 0; i < order.size(); ++i) {
      sc[i] = codes[order[i]];
      scnt[i] = code_counts[order[i]];
    }
    // RoundInt((total - na) * 0.99f): the product in f32, the rounding in f64
    const float prod = (float)(total_sample_cnt - (int64_t)na_cnt) * 0.99f;
    const int32_t cut_cnt = (int32_t)((double)prod + 0.5);
    int32_t distinct_cnt = (int32_t)sc.size() + (na_cnt > 0 ? 1 : 0);
    const int32_t mb = std::min(distinct_cnt, max_bin);
    b2c.push_back(-1);
    cnt_in_bin.push_back(0);
    num_bin = 1;
    int32_t used_cnt = 0;
    size_t cur = 0;
    while (cur < sc.size() && (used_cnt < cut_cnt || num_bin < mb)) {
      if (scnt[cur] < min_data_in_bin && cur > 1) break;
      b2c.push_back(sc[cur]);
      used_cnt += scnt[cur];
      cnt_in_bin.push_back(scnt[cur]);
      ++num_bin;
      ++cur;
    }
    missing = (cur == sc.size() && na_cnt == 0) ? 0 : 2;
    cnt_in_bin[0] = (int32_t)(total_sample_cnt - used_cnt);
  }
  bool is_trivial = num_bin <= 1;
  if (!is_trivial && pre_filter) {
    // need_filter for categorical bins (bin.rs:309-317): only two-bin features can be filtered
    bool filt = false;
    if (cnt_in_bin.size() <= 2) {
      filt = true;
      for (size_t i = 0; i + 1 < cnt_in_bin.size(); ++i)
        if (cnt_in_bin[i] >= min_split_data && (int32_t)total_sample_cnt - cnt_in_bin[i] >= min_split_data)
          filt = false;
    }
    if (filt) is_trivial = true;
  }
  int32_t default_bin = 0, mfb = 0;
  double sparse_rate = 1.0;
  if (!is_trivial) {
    for (int32_t b = 1; b < num_bin; ++b)  // value_to_bin(0.0): the bin of code 0, else 0
      if (b2c[(size_t)b] == 0) default_bin = b;
    size_t am = 0;
    for (size_t i = 1; i < cnt_in_bin.size(); ++i)
      if (cnt_in_bin[i] > cnt_in_bin[am]) am = i;
    mfb = (int32_t)am;
    double max_sparse_rate = (double)cnt_in_bin[(size_t)mfb] / (double)total_sample_cnt;
    if (mfb != default_bin && max_sparse_rate < K_SPARSE_THRESHOLD) mfb = default_bin;
    sparse_rate = (double)cnt_in_bin[(size_t)mfb] / (double)total_sample_cnt;
  }
  if (num_bin > cap) return -1;
  for (int32_t i = 0; i < num_bin && i < (int32_t)b2c.size(); ++i) bin_to_category[i] = b2c[(size_t)i];
  meta_out[0] = missing;
  meta_out[1] = is_trivial ? 1 : 0;
  meta_out[2] = default_bin;
  meta_out[3] = mfb;
  dmeta_out[0] = min_val;
  dmeta_out[1] = max_val;
  dmeta_out[2] = sparse_rate;
  return num_bin;
}

// Stored group bins of one categorical single-feature group (dataset.rs:633-685 with the
// categorical BinMapper::value_to_bin, bin.rs:558-589: NaN and negative codes go to bin 0, codes
// without a bin too).
void bk_values_to_group_bins_categorical(const double* col, int64_t n, int64_t stride, const int32_t* bin_to_category,
                                         int32_t num_bin, int32_t most_freq_bin, uint8_t* out) {
  for (int64_t i = 0; i < n; ++i) {
    const double v = col[i * stride];
    int32_t bin = 0;
    if (!std::isnan(v)) {
      const int32_t code = cat_code(v);
      if (code >= 0)
        for (int32_t b = 1; b < num_bin; ++b)
          if (bin_to_category[b] == code) {
            bin = b;
            break;
          }
    }
    out[i] = (uint8_t)(bin == most_freq_bin ? 0 : bin + 1 - (most_freq_bin == 0 ? 1 : 0));
  }
}

// Stored group bins of one single-feature dense group (dataset.rs:633-685 fill_dense, with
// BinMapper::value_to_bin of bin.rs:558-589): bin == most_freq_bin is stored as 0, other bins
// as bin + 1 - (most_freq_bin == 0). Column of `n` values with stride `stride` doubles.
void bk_values_to_group_bins(const double* col, int64_t n, int64_t stride, const double* upper_bounds,
                             int32_t num_bin, int32_t missing_type, int32_t most_freq_bin, uint8_t* out) {
  int32_t rr = num_bin - 1 - (missing_type == 2 ? 1 : 0);
  for (int64_t i = 0; i < n; ++i) {
    double v = col[i * stride];
    int32_t bin;
    if (std::isnan(v) && missing_type == 2) {
      bin = num_bin - 1;
    } else {
      if (std::isnan(v)) v = 0.0;
      int32_t l = 0, r = rr;
      while (l < r) {
        int32_t mid = (r + l - 1) / 2;
        if (v <= upper_bounds[mid]) r = mid;
        else l = mid + 1;
      }
      bin = l;
    }
    int32_t stored;
    if (bin == most_freq_bin) stored = 0;
    else stored = bin + 1 - (most_freq_bin == 0 ? 1 : 0);
    out[i] = (uint8_t)stored;
  }
}

}  // extern "C"

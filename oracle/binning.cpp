// ORACLE — test infrastructure only. The oracle's own dataset preparation for dense numerical
// data, restated from bankai-lightgbm's io/ (the product library's binning is not used here, so
// the CPU reference arm and the parity tests bin their rows independently of the code under
// test):
//   - the bin-construction row sample: create_sample_indices (io/sample.rs:16-19) with the
//     LCG's Random::sample (utils/random.rs:52-76);
//   - BinMapper::find_bin for numerical features without forced bounds (io/bin.rs:342-554),
//     with GreedyFindBin (io/bin.rs:51-137), FindBinWithZeroAsOneBin (io/bin.rs:228-297) and
//     NeedFilter (io/bin.rs:300-319);
//   - BinMapper::value_to_bin (io/bin.rs:558-589) and the stored group bin of a dense
//     single-feature group (io/dataset.rs:633-685): a row whose bin is the most frequent bin
//     stores 0, any other row stores bin + 1 - (most_freq_bin == 0).
//
// Compiled with -ffp-contract=off: the bound arithmetic rounds like the reference's.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <set>
#include <thread>
#include <vector>

namespace orcbin {

const double kZero = (double)1e-35f;  // meta.rs:4 kZeroThreshold
const double kSparse = 0.7;           // bin.rs:9 kSparseThreshold
const double kInf = std::numeric_limits<double>::infinity();

// Common::GetDoubleUpperBound / CheckDoubleEqualOrdered (bin.rs:39-48)
double up(double a) { return std::nextafter(a, kInf); }
bool same_ordered(double a, double b) { return b <= up(a); }

// A sorted run of distinct sample values with their counts.
struct Runs {
  std::vector<double> v;
  std::vector<int32_t> c;
};

// Appends `val` unless it rounds onto the last bound (bin.rs:69-72, :126-131).
void push_bound(std::vector<double>& ub, double val) {
  if (ub.empty() || !same_ordered(ub.back(), val)) ub.push_back(val);
}

// GreedyFindBin (bin.rs:51-137) over runs [lo, hi).
std::vector<double> greedy(const Runs& r, size_t lo, size_t hi, int32_t max_bin, int64_t total, int32_t min_in_bin) {
  const size_t nd = hi - lo;
  const double* v = r.v.data() + lo;
  const int32_t* c = r.c.data() + lo;
  std::vector<double> ub;
  if ((int64_t)nd <= (int64_t)max_bin) {
    // few distinct values: a bound between neighbours once a bin holds min_data_in_bin
    int32_t acc = 0;
    for (size_t i = 0; i + 1 < nd; ++i) {
      acc += c[i];
      if (acc < min_in_bin) continue;
      const size_t before = ub.size();
      push_bound(ub, up((v[i] + v[i + 1]) / 2.0));
      if (ub.size() != before) acc = 0;
    }
    ub.push_back(kInf);
    return ub;
  }
  if (min_in_bin > 0) max_bin = std::max(1, std::min(max_bin, (int32_t)(total / (int64_t)min_in_bin)));
  // values holding at least a mean bin's worth of samples get a bin of their own
  double mean = (double)total / (double)max_bin;
  std::vector<char> big(nd, 0);
  int32_t rest_bins = max_bin, rest_cnt = (int32_t)total;
  for (size_t i = 0; i < nd; ++i)
    if ((double)c[i] >= mean) {
      big[i] = 1;
      --rest_bins;
      rest_cnt -= c[i];
    }
  mean = (double)rest_cnt / (double)rest_bins;
  std::vector<double> hi_v((size_t)max_bin, kInf), lo_v((size_t)max_bin, kInf);
  size_t nb = 0;
  lo_v[0] = v[0];
  int32_t acc = 0;
  for (size_t i = 0; i + 1 < nd; ++i) {
    if (!big[i]) rest_cnt -= c[i];
    acc += c[i];
    const bool cut = big[i] || (double)acc >= mean || (big[i + 1] && (double)acc >= std::max(1.0, mean * 0.5));
    if (!cut) continue;
    hi_v[nb] = v[i];
    ++nb;
    lo_v[nb] = v[i + 1];
    if ((int32_t)nb >= max_bin - 1) break;
    acc = 0;
    if (!big[i]) {
      --rest_bins;
      mean = (double)rest_cnt / (double)rest_bins;
    }
  }
  ++nb;
  for (size_t i = 0; i + 1 < nb; ++i) push_bound(ub, up((hi_v[i] + lo_v[i + 1]) / 2.0));
  ub.push_back(kInf);
  return ub;
}

// FindBinWithZeroAsOneBin without forced bounds (bin.rs:228-297): negative values, a bin of
// zeros (bounded by -kZeroThreshold / +kZeroThreshold), positive values.
std::vector<double> zero_as_one_bin(const Runs& r, int32_t max_bin, int64_t total, int32_t min_in_bin) {
  const size_t nd = r.v.size();
  int32_t neg = 0, zero = 0, pos = 0;
  size_t first_nonneg = nd, first_pos = nd;
  for (size_t i = 0; i < nd; ++i) {
    const double x = r.v[i];
    if (x <= -kZero) neg += r.c[i];
    else if (x > kZero) pos += r.c[i];
    else zero += r.c[i];
    if (first_nonneg == nd && x > -kZero) first_nonneg = i;
  }
  for (size_t i = first_nonneg; i < nd; ++i)
    if (r.v[i] > kZero) {
      first_pos = i;
      break;
    }
  std::vector<double> ub;
  if (first_nonneg > 0 && max_bin > 1) {
    const int32_t left_bins =
        std::max(1, (int32_t)((double)neg / ((double)total - (double)zero) * (double)(max_bin - 1)));
    ub = greedy(r, 0, first_nonneg, left_bins, neg, min_in_bin);
    if (!ub.empty()) ub.back() = -kZero;
  }
  const int32_t right_bins = max_bin - 1 - (int32_t)ub.size();
  if (first_pos < nd && right_bins > 0) {
    std::vector<double> right = greedy(r, first_pos, nd, right_bins, pos, min_in_bin);
    ub.push_back(kZero);
    ub.insert(ub.end(), right.begin(), right.end());
  } else {
    ub.push_back(kInf);
  }
  return ub;
}

struct Mapper {
  std::vector<double> bounds;
  int32_t missing = 0;  // 0 none, 1 zero, 2 NaN
  int32_t default_bin = 0, mfb = 0;
  bool trivial = false;
  double min_val = 0, max_val = 0, sparse_rate = 1.0;

  // BinMapper::value_to_bin (bin.rs:558-589), numerical
  uint32_t bin_of(double x) const {
    const int32_t nb = (int32_t)bounds.size();
    if (std::isnan(x)) {
      if (missing == 2) return (uint32_t)(nb - 1);
      x = 0.0;
    }
    int32_t l = 0, r = nb - 1 - (missing == 2 ? 1 : 0);
    while (l < r) {
      const int32_t m = (r + l - 1) / 2;
      if (x <= bounds[(size_t)m]) r = m;
      else l = m + 1;
    }
    return (uint32_t)l;
  }

  // BinMapper::find_bin (bin.rs:342-554), numerical, no forced bounds. `vals`: the sampled values
  // with |v| > kZeroThreshold or NaN (zeros are implied by total_cnt).
  void find(std::vector<double> vals, int64_t total_cnt, int32_t max_bin, int32_t min_in_bin, int32_t filter_cnt,
            bool pre_filter, bool use_missing, bool zero_as_missing) {
    size_t finite = 0;
    for (double x : vals)
      if (!std::isnan(x)) vals[finite++] = x;
    const int64_t na = (int64_t)vals.size() - (int64_t)finite;
    int64_t na_cnt = 0;
    if (!use_missing) missing = 0;
    else if (zero_as_missing) missing = 1;
    else if (na == 0) missing = 0;
    else {
      missing = 2;
      na_cnt = na;
    }
    vals.resize(finite);
    const int32_t zeros = (int32_t)(total_cnt - (int64_t)finite - na_cnt);
    std::stable_sort(vals.begin(), vals.end());
    // distinct values (bin.rs:393-428): neighbours within one ulp merge into the larger one; the
    // implied zeros enter where the sign changes
    Runs r;
    auto add = [&](double x, int32_t cnt) {
      r.v.push_back(x);
      r.c.push_back(cnt);
    };
    if (finite == 0 || (vals[0] > 0.0 && zeros > 0)) add(0.0, zeros);
    for (size_t i = 0; i < finite; ++i) {
      if (i > 0 && same_ordered(vals[i - 1], vals[i])) {
        r.v.back() = vals[i];
        r.c.back() += 1;
        continue;
      }
      if (i > 0 && vals[i - 1] < 0.0 && vals[i] > 0.0) add(0.0, zeros);
      add(vals[i], 1);
    }
    if (finite > 0 && vals[finite - 1] < 0.0 && zeros > 0) add(0.0, zeros);
    min_val = r.v.front();
    max_val = r.v.back();
    if (missing == 2) {
      bounds = zero_as_one_bin(r, max_bin - 1, total_cnt - na_cnt, min_in_bin);
      bounds.push_back(2.0);  // upstream stores MissingType::NaN (= 2) as the NaN bin's bound
    } else {
      bounds = zero_as_one_bin(r, max_bin, total_cnt, min_in_bin);
      if (missing == 1 && bounds.size() == 2) missing = 0;
    }
    const int32_t nb = (int32_t)bounds.size();
    std::vector<int32_t> in_bin((size_t)nb, 0);
    size_t b = 0;
    for (size_t i = 0; i < r.v.size(); ++i) {
      while (r.v[i] > bounds[b] && (int32_t)b < nb - 1) ++b;
      in_bin[b] += r.c[i];
    }
    if (missing == 2) in_bin.back() = (int32_t)na_cnt;
    trivial = nb <= 1;
    if (!trivial && pre_filter) {
      // NeedFilter (bin.rs:300-319): trivial unless some cut leaves filter_cnt samples each side
      bool keep = false;
      int32_t left = 0;
      for (int32_t i = 0; i + 1 < nb && !keep; ++i) {
        left += in_bin[(size_t)i];
        keep = left >= filter_cnt && (int32_t)total_cnt - left >= filter_cnt;
      }
      trivial = !keep;
    }
    if (trivial) {
      sparse_rate = 1.0;
      return;
    }
    default_bin = (int32_t)bin_of(0.0);
    mfb = (int32_t)(std::max_element(in_bin.begin(), in_bin.end()) - in_bin.begin());  // first maximum
    if (mfb != default_bin && (double)in_bin[(size_t)mfb] / (double)total_cnt < kSparse) mfb = default_bin;
    sparse_rate = (double)in_bin[(size_t)mfb] / (double)total_cnt;
  }

  // io/dataset.rs:633-685 — the stored bin of one value in its own dense group
  uint8_t stored(double x) const {
    uint32_t b = bin_of(x);
    if ((int32_t)b == mfb) return 0;
    return (uint8_t)(b + (mfb == 0 ? 0u : 1u));
  }
};

// Random::sample (utils/random.rs:52-76) with the LCG of utils/random.rs:17-50.
std::vector<int64_t> lcg_sample(int64_t n, int64_t k, int32_t seed) {
  uint32_t x = (uint32_t)seed;
  auto i16 = [&]() -> int32_t {
    x = x * 214013u + 2531011u;
    return (int32_t)((x >> 16) & 0x7fffu);
  };
  auto i31 = [&]() -> int32_t {
    x = x * 214013u + 2531011u;
    return (int32_t)(x & 0x7fffffffu);
  };
  std::vector<int64_t> out;
  if (k > n || k <= 0) return out;
  if (k == n) {
    for (int64_t i = 0; i < n; ++i) out.push_back(i);
    return out;
  }
  if (k > 1 && (double)k > (double)n / std::log2((double)k)) {
    for (int64_t i = 0; i < n; ++i) {
      const double prob = (double)(k - (int64_t)out.size()) / (double)(n - i);
      const float f = (float)i16() / 32768.0f;
      if ((double)f < prob) out.push_back(i);
    }
    return out;
  }
  std::set<int64_t> s;
  for (int64_t r = n - k; r < n; ++r) {
    const int64_t v = i31() % (r + 1);
    if (!s.insert(v).second) s.insert(r);
  }
  out.assign(s.begin(), s.end());
  return out;
}

template <typename T>
void run_threads(int threads, int64_t count, const T& fn) {
  threads = std::max(1, std::min<int>(threads, (int)std::max<int64_t>(count, 1)));
  std::vector<std::thread> ws;
  for (int t = 0; t < threads; ++t)
    ws.emplace_back([&, t] {
      for (int64_t i = t; i < count; i += threads) fn(i);
    });
  for (auto& w : ws) w.join();
}

}  // namespace orcbin

extern "C" {

// The oracle's dense dataset: bin mappers found on the LCG row sample (io/sample.rs) and every
// stored bin, for a row-major float32 matrix X [n][ncol].
//   meta_out [ncol][4]: missing type, trivial flag, default bin, most frequent bin;
//   nbin_out [ncol]; bounds_out [ncol][cap] upper bounds;
//   bins_out [ncol][n] stored bins (written for non-trivial columns only; may be NULL).
// Returns 0, or -1 if a column needs more than `cap` bounds.
int32_t orc_bin_dense_f32(const float* X, int64_t n, int32_t ncol, int32_t max_bin, int32_t min_data_in_bin,
                          int32_t min_data_in_leaf, int64_t bin_construct_sample_cnt, int32_t data_random_seed,
                          int32_t threads, int32_t cap, int32_t* meta_out, int32_t* nbin_out, double* bounds_out,
                          uint8_t* bins_out) {
  using namespace orcbin;
  const std::vector<int64_t> rows = lcg_sample(n, std::min(n, bin_construct_sample_cnt), data_random_seed);
  const int64_t sample_cnt = (int64_t)rows.size();
  // io/dataset.rs — filter_cnt = min_data_in_leaf * sample_cnt / num_data
  const int32_t filter_cnt = (int32_t)((double)min_data_in_leaf * (double)sample_cnt / (double)n);
  std::vector<Mapper> maps((size_t)ncol);
  std::vector<int> too_many((size_t)ncol, 0);
  run_threads(threads, ncol, [&](int64_t col) {
    std::vector<double> vals;
    vals.reserve((size_t)sample_cnt);
    for (int64_t r : rows) {
      const double x = (double)X[(size_t)r * (size_t)ncol + (size_t)col];
      if (std::isnan(x) || std::fabs(x) > kZero) vals.push_back(x);
    }
    Mapper& m = maps[(size_t)col];
    m.find(std::move(vals), sample_cnt, max_bin, min_data_in_bin, filter_cnt, true, true, false);
    if ((int32_t)m.bounds.size() > cap) too_many[(size_t)col] = 1;
  });
  for (int32_t c = 0; c < ncol; ++c)
    if (too_many[(size_t)c]) return -1;
  for (int32_t c = 0; c < ncol; ++c) {
    const Mapper& m = maps[(size_t)c];
    meta_out[4 * c + 0] = m.missing;
    meta_out[4 * c + 1] = m.trivial ? 1 : 0;
    meta_out[4 * c + 2] = m.default_bin;
    meta_out[4 * c + 3] = m.mfb;
    nbin_out[c] = (int32_t)m.bounds.size();
    std::memcpy(bounds_out + (size_t)c * (size_t)cap, m.bounds.data(), sizeof(double) * m.bounds.size());
  }
  if (!bins_out) return 0;
  // stored bins, row blocks in parallel (each thread reads whole rows of X once)
  const int64_t block = 4096;
  const int64_t nblocks = (n + block - 1) / block;
  run_threads(threads, nblocks, [&](int64_t b) {
    const int64_t r0 = b * block, r1 = std::min(n, r0 + block);
    for (int32_t c = 0; c < ncol; ++c) {
      const Mapper& m = maps[(size_t)c];
      if (m.trivial) continue;
      uint8_t* out = bins_out + (size_t)c * (size_t)n;
      for (int64_t r = r0; r < r1; ++r) out[r] = m.stored((double)X[(size_t)r * (size_t)ncol + (size_t)c]);
    }
  });
  return 0;
}

// BinMapper::find_bin (numerical) on given sample values, for the pins against the reference's
// golden bin mappers. vals: the sampled values (all of them; zeros are dropped here). meta_out:
// missing type, trivial, default bin, most frequent bin; dmeta_out: min, max, sparse rate.
// Returns num_bin, or -1 above `cap`.
int32_t orc_find_bin(const double* sample, int64_t count, int64_t total_sample_cnt, int32_t max_bin,
                     int32_t min_data_in_bin, int32_t filter_cnt, int32_t pre_filter, int32_t use_missing,
                     int32_t zero_as_missing, double* bounds_out, int32_t cap, int32_t* meta_out, double* dmeta_out) {
  using namespace orcbin;
  std::vector<double> vals;
  for (int64_t i = 0; i < count; ++i)
    if (std::isnan(sample[i]) || std::fabs(sample[i]) > kZero) vals.push_back(sample[i]);
  Mapper m;
  m.find(std::move(vals), total_sample_cnt, max_bin, min_data_in_bin, filter_cnt, pre_filter != 0, use_missing != 0,
         zero_as_missing != 0);
  if ((int32_t)m.bounds.size() > cap) return -1;
  std::memcpy(bounds_out, m.bounds.data(), sizeof(double) * m.bounds.size());
  meta_out[0] = m.missing;
  meta_out[1] = m.trivial ? 1 : 0;
  meta_out[2] = m.default_bin;
  meta_out[3] = m.mfb;
  dmeta_out[0] = m.min_val;
  dmeta_out[1] = m.max_val;
  dmeta_out[2] = m.sparse_rate;
  return (int32_t)m.bounds.size();
}

// The LCG row sample of bin construction (io/sample.rs:16-19): k sorted row ids of n.
int64_t orc_sample_rows(int64_t n, int64_t k, int32_t seed, int64_t* out) {
  const std::vector<int64_t> s = orcbin::lcg_sample(n, k, seed);
  std::copy(s.begin(), s.end(), out);
  return (int64_t)s.size();
}

}  // extern "C"

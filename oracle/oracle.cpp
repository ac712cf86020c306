// ORACLE — test infrastructure only.
//
// A plain C++ CPU restatement of bankai-lightgbm's tree-learner hot path, used as the parity
// oracle of the GB300 learner and as the timed CPU baseline ("port"). Nothing in the product
// library links, loads or calls this file; only tests, the smoke check and the CPU-baseline leg
// of bench.py do.
//
// Every routine follows one reference routine, cited as path:line inside bankai-lightgbm
// (crates/lgbm-core/src/...). Floating-point expressions are written in the reference's
// evaluation order and the file is compiled with -ffp-contract=off, so `a * b + c` is never
// fused behind our back; the one place the reference fuses on aarch64 (`madd`,
// utils/common.rs:207-216) is an explicit runtime switch (`fused_madd`).
//
// Scope: dense numerical single-feature groups (the layout produced by Dataset::from_dense for
// dense data), full histogram pool, no monotone constraints / CEGB / forced splits / extra trees /
// linear trees / categorical features.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

namespace orc {

// meta.rs:7 — kEpsilon is a float literal (1e-15f) widened to double.
static const double EPS = (double)1e-15f;
// meta.rs:4 — kZeroThreshold = 1e-35f widened to double.
static const double K_ZERO_THRESHOLD = (double)1e-35f;
static const double K_MIN_SCORE = -std::numeric_limits<double>::infinity();

enum Missing : int32_t { MISSING_NONE = 0, MISSING_ZERO = 1, MISSING_NAN = 2 };

// utils/common.rs:207-216 — `a * b + c`, fused only where the reference build fuses (aarch64).
static inline double madd(double a, double b, double c, bool fused) {
  if (fused) return std::fma(a, b, c);
  double p = a * b;
  return p + c;
}

// ---------------------------------------------------------------------------------------------
// std::mt19937 and the libc++ distributions (treelearner/gradient_discretizer/mt19937.rs:32-128)
// ---------------------------------------------------------------------------------------------
struct Mt19937 {
  uint32_t st[624];
  int idx;
  explicit Mt19937(uint32_t seed = 5489u) { seed_with(seed); }
  void seed_with(uint32_t seed) {
    st[0] = seed;
    for (int i = 1; i < 624; ++i) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
    idx = 624;
  }
  void twist() {
    for (int i = 0; i < 624; ++i) {
      uint32_t y = (st[i] & 0x80000000u) | (st[(i + 1) % 624] & 0x7fffffffu);
      uint32_t nx = st[(i + 397) % 624] ^ (y >> 1);
      if (y & 1u) nx ^= 0x9908b0dfu;
      st[i] = nx;
    }
    idx = 0;
  }
  uint32_t next_u32() {
    if (idx >= 624) twist();
    uint32_t y = st[idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  // mt19937.rs:95-101 — libc++ generate_canonical<double,53>: two draws, low word first.
  double uniform_real_01() {
    double g1 = (double)next_u32();
    double g2 = (double)next_u32();
    double rp = 4294967296.0;
    double sp = g1 + g2 * rp;
    return sp / (rp * rp);
  }
  // mt19937.rs:109-128 — libc++ uniform_int_distribution<int>(0, n) with rejection.
  uint32_t uniform_int_inclusive(uint32_t n) {
    uint32_t rp = n + 1u;
    if (rp == 1u) return 0u;
    if (rp == 0u) return next_u32();
    int lz = __builtin_clz(rp);
    uint32_t w = 32u - (uint32_t)lz - 1u;
    if (rp & (0xffffffffu >> (32u - w))) w += 1u;
    uint32_t mask = w >= 32u ? 0xffffffffu : ((1u << w) - 1u);
    for (;;) {
      uint32_t u = next_u32() & mask;
      if (u < rp) return u;
    }
  }
};

// gradient_discretizer/mod.rs:19-29 — Threading::BlockInfo.
static void block_info(size_t num_threads, size_t cnt, size_t min_cnt, size_t* n_block, size_t* size) {
  size_t nt = num_threads < 1 ? 1 : num_threads;
  size_t mc = min_cnt < 1 ? 1 : min_cnt;
  size_t nb = std::min(nt, (cnt + mc - 1) / mc);
  if (nb > 1) {
    size_t s = (cnt + nb - 1) / nb;
    *n_block = nb;
    *size = (s + 31) / 32 * 32;
  } else {
    *n_block = nb;
    *size = cnt;
  }
}

// Rust `f64 as i8`: saturating, NaN -> 0.
static inline int8_t sat_i8(double v) {
  if (std::isnan(v)) return 0;
  if (v >= 127.0) return 127;
  if (v <= -128.0) return -128;
  return (int8_t)(int)std::trunc(v);
}

// gradient_discretizer/mod.rs:35-217 — GradientDiscretizer.
struct Discretizer {
  std::vector<int16_t> packed;
  int bins = 4;
  bool constant_hessian = false;
  double gscale = 0.0, hscale = 0.0;
  bool stochastic = false;
  std::vector<double> grand, hrand;
  Mt19937 use_start;
  bool fused = false;

  void init(size_t n, int b, bool const_hess, bool fused_madd) {
    packed.assign(n, 0);
    bins = b;
    constant_hessian = const_hess;
    fused = fused_madd;
  }
  // mod.rs:87-106
  void init_stochastic(uint32_t seed, size_t num_threads) {
    size_t n = packed.size();
    use_start.seed_with(seed);
    grand.assign(n, 0.0);
    hrand.assign(n, 0.0);
    size_t threads = num_threads < 1 ? 1 : num_threads;
    size_t nb, bs;
    block_info(threads, n, 512, &nb, &bs);
    for (size_t b = 0; b < nb; ++b) {
      size_t start = b * bs, end = std::min(start + bs, n);
      Mt19937 ge(seed + (uint32_t)b);
      Mt19937 he(seed + (uint32_t)b + (uint32_t)threads);
      for (size_t i = start; i < end; ++i) {
        grand[i] = ge.uniform_real_01();
        hrand[i] = he.uniform_real_01();
      }
    }
    stochastic = true;
  }
  // mod.rs:134-165 — returns false on the refused cases (previous state kept).
  bool update_scales(const float* g, const float* h, double* inv_g, double* inv_h) {
    size_t n = packed.size();
    float max_g = 0.0f, max_h = 0.0f;
    for (size_t i = 0; i < n; ++i) {
      if (!std::isfinite(g[i]) || !std::isfinite(h[i]) || h[i] < 0.0f) return false;
    }
    for (size_t i = 0; i < n; ++i) max_g = std::max(max_g, std::fabs(g[i]));
    for (size_t i = 0; i < n; ++i) max_h = std::max(max_h, h[i]);
    if (max_g == 0.0f || (!constant_hessian && max_h == 0.0f)) return false;
    gscale = (double)max_g / (double)(bins / 2);
    hscale = constant_hessian ? (double)max_h : (double)max_h / (double)bins;
    *inv_g = 1.0 / gscale;
    *inv_h = 1.0 / hscale;
    return true;
  }
  // mod.rs:116-130
  bool discretize_nearest(const float* g, const float* h) {
    double ig, ih;
    if (!update_scales(g, h, &ig, &ih)) return false;
    for (size_t i = 0; i < packed.size(); ++i) {
      double gv = (double)g[i];
      double off = gv >= 0.0 ? 0.5 : -0.5;
      int8_t gi = sat_i8(madd(gv, ig, off, fused));
      int8_t hi = constant_hessian ? 1 : sat_i8(madd((double)h[i], ih, 0.5, fused));
      packed[i] = (int16_t)(((int)gi << 8) | (int)(uint8_t)hi);
    }
    return true;
  }
  // mod.rs:172-201
  bool discretize_stochastic(const float* g, const float* h) {
    if (!stochastic) return false;
    double ig, ih;
    if (!update_scales(g, h, &ig, &ih)) return false;
    size_t n = packed.size();
    size_t start = use_start.uniform_int_inclusive((uint32_t)n);
    for (size_t i = 0; i < n; ++i) {
      size_t pos = (i + start) % n;
      double gv = (double)g[i];
      double noise = grand[pos];
      double sn = gv >= 0.0 ? noise : -noise;
      int8_t gi = sat_i8(madd(gv, ig, sn, fused));
      int8_t hi = constant_hessian ? 1 : sat_i8(madd((double)h[i], ih, hrand[pos], fused));
      packed[i] = (int16_t)(((int)gi << 8) | (int)(uint8_t)hi);
    }
    return true;
  }
};

// ---------------------------------------------------------------------------------------------
// Split search (treelearner/feature_histogram.rs)
// ---------------------------------------------------------------------------------------------
struct Params {
  double l1 = 0, l2 = 0, max_delta = 0, smooth = 0;
  int32_t min_data = 20;
  double min_hess = 1e-3;
  double min_gain = 0;
  bool fused = false;
  // CatParams (feature_histogram.rs:1146-1163), config/auto.rs:214-218 defaults
  double cat_smooth = 10.0, cat_l2 = 10.0;
  int32_t max_cat_threshold = 32, max_cat_to_onehot = 4, min_data_per_group = 100;
};

struct FeatureMeta {
  int32_t num_bin, missing, offset, default_bin, mfb;
  double penalty;
  int32_t real;
  int32_t categorical = 0;  // BinType::Categorical
};

struct SplitInfo {
  int32_t feature = -1;
  uint32_t threshold = 0;
  int32_t left_count = 0, right_count = 0;
  double left_output = 0, right_output = 0, gain = K_MIN_SCORE;
  double lsg = 0, lsh = 0, rsg = 0, rsh = 0;
  int64_t lint = 0, rint = 0;
  bool default_left = true;
  std::vector<uint32_t> cat_bins;  // categorical: the bins that go left (cat_threshold)
  // split_info.rs:104-121
  bool better_than(const SplitInfo& o) const {
    double a = gain, b = o.gain;
    if (a != b) return a > b;
    int32_t fa = feature == -1 ? INT32_MAX : feature;
    int32_t fb = o.feature == -1 ? INT32_MAX : o.feature;
    return fa < fb;
  }
};

static inline double sgn(double x) { return (double)((int)(x > 0.0) - (int)(x < 0.0)); }
static inline int32_t round_int(double x) {  // feature_histogram.rs:66 — (x + 0.5) as i32
  double v = x + 0.5;
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0) return INT32_MAX;
  if (v <= -2147483648.0) return INT32_MIN;
  return (int32_t)v;
}
static inline double threshold_l1(double s, double l1) {  // :72-75
  double reg = std::max(std::fabs(s) - l1, 0.0);
  return sgn(s) * reg;
}

struct Flags { bool l1, mx, sm; };

// :79-104
static double leaf_output(const Flags& F, double sg, double sh, const Params& p, int32_t n, double parent) {
  double ret;
  if (F.l1) ret = -threshold_l1(sg, p.l1) / (sh + p.l2);
  else ret = -sg / (sh + p.l2);
  if (F.mx && p.max_delta > 0.0 && std::fabs(ret) > p.max_delta) ret = sgn(ret) * p.max_delta;
  if (F.sm) {
    double nn = (double)n;
    double a = nn / p.smooth;
    double t1 = ret * a;
    t1 = t1 / (a + 1.0);
    double t2 = parent / (a + 1.0);
    ret = t1 + t2;
  }
  return ret;
}

// :127-144
static double leaf_gain_given_output(bool l1, double sg, double sh, const Params& p, double out) {
  double g = l1 ? threshold_l1(sg, p.l1) : sg;
  double hl = sh + p.l2;
  double q = hl * out;
  q = q * out;
  return -madd(2.0 * g, out, q, p.fused);
}

// :148-176
static double leaf_gain(const Flags& F, double sg, double sh, const Params& p, int32_t n, double parent) {
  if (!F.mx && !F.sm) {
    if (F.l1) {
      double s = threshold_l1(sg, p.l1);
      return (s * s) / (sh + p.l2);
    }
    return (sg * sg) / (sh + p.l2);
  }
  double out = leaf_output(F, sg, sh, p, n, parent);
  return leaf_gain_given_output(F.l1, sg, sh, p, out);
}

// simd.rs:6-8 — gl*gl/(hl+l2) + gr*gr/(hr+l2), each operation rounded separately.
static double split_gain(double gl, double hl, double gr, double hr, double l2) {
  double a = gl * gl;
  a = a / (hl + l2);
  double b = gr * gr;
  b = b / (hr + l2);
  return a + b;
}

static double gains(const Flags& F, const Params& p, double slg, double slh, double srg, double srh, int32_t lc,
                    int32_t rc, double parent) {
  if (!F.l1 && !F.mx && !F.sm) return split_gain(slg, slh, srg, srh, p.l2);
  double a = leaf_gain(F, slg, slh, p, lc, parent);
  double b = leaf_gain(F, srg, srh, p, rc, parent);
  return a + b;
}

// feature_histogram.rs:363-663 — FindBestThresholdSequentially (float), no RAND, no MC.
static bool sequential(const Flags& F, bool REV, bool SKIP, bool NA, const double* hist, const FeatureMeta& m,
                       const Params& p, double sum_g, double sum_h, int32_t num_data, double min_gain_shift,
                       double parent, SplitInfo* out) {
  const int32_t offset = m.offset;
  bool is_splittable = false;
  double best_slg = NAN, best_slh = NAN, best_gain = K_MIN_SCORE;
  int32_t best_lc = 0;
  uint32_t best_th = (uint32_t)m.num_bin;
  double cnt_factor = (double)num_data / sum_h;
  auto G = [&](int t) { return hist[(size_t)t << 1]; };
  auto H = [&](int t) { return hist[((size_t)t << 1) + 1]; };
  if (REV) {
    double srg = 0.0, srh = EPS;
    int32_t rc = 0;
    int t = m.num_bin - 1 - offset - (NA ? 1 : 0);
    int t_end = 1 - offset;
    for (; t >= t_end; --t) {
      if (SKIP && (t + offset) == m.default_bin) continue;
      double g = G(t), h = H(t);
      int32_t cnt = round_int(h * cnt_factor);
      srg += g;
      srh += h;
      rc += cnt;
      if (rc < p.min_data || srh < p.min_hess) continue;
      int32_t lc = num_data - rc;
      if (lc < p.min_data) break;
      double slh = sum_h - srh;
      if (slh < p.min_hess) break;
      double slg = sum_g - srg;
      double cg = gains(F, p, slg, slh, srg, srh, lc, rc, parent);
      if (cg <= min_gain_shift) continue;
      is_splittable = true;
      if (cg > best_gain) {
        best_lc = lc;
        best_slg = slg;
        best_slh = slh;
        best_th = (uint32_t)(t - 1 + offset);
        best_gain = cg;
      }
    }
  } else {
    double slg = 0.0, slh = EPS;
    int32_t lc = 0;
    int t = 0;
    int t_end = m.num_bin - 2 - offset;
    if (NA && offset == 1) {
      slg = sum_g;
      slh = sum_h - EPS;
      lc = num_data;
      for (int i = 0; i < m.num_bin - offset; ++i) {
        double g = G(i), h = H(i);
        int32_t cnt = round_int(h * cnt_factor);
        slg -= g;
        slh -= h;
        lc -= cnt;
      }
      t = -1;
    }
    for (; t <= t_end; ++t) {
      if (SKIP && (t + offset) == m.default_bin) continue;
      if (t >= 0) {
        slg += G(t);
        slh += H(t);
        lc += round_int(H(t) * cnt_factor);
      }
      if (lc < p.min_data || slh < p.min_hess) continue;
      int32_t rc = num_data - lc;
      if (rc < p.min_data) break;
      double srh = sum_h - slh;
      if (srh < p.min_hess) break;
      double srg = sum_g - slg;
      double cg = gains(F, p, slg, slh, srg, srh, lc, rc, parent);
      if (cg <= min_gain_shift) continue;
      is_splittable = true;
      if (cg > best_gain) {
        best_lc = lc;
        best_slg = slg;
        best_slh = slh;
        best_th = (uint32_t)(t + offset);
        best_gain = cg;
      }
    }
  }
  if (is_splittable && best_gain > out->gain + min_gain_shift) {
    out->threshold = best_th;
    out->left_output = leaf_output(F, best_slg, best_slh, p, best_lc, parent);
    out->left_count = best_lc;
    out->lsg = best_slg;
    out->lsh = best_slh - EPS;
    out->right_output = leaf_output(F, sum_g - best_slg, sum_h - best_slh, p, num_data - best_lc, parent);
    out->right_count = num_data - best_lc;
    out->rsg = sum_g - best_slg;
    out->rsh = sum_h - best_slh - EPS;
    out->gain = best_gain - min_gain_shift;
    out->default_left = REV;
  }
  return is_splittable;
}

// feature_histogram.rs:219-357 — FindBestThreshold (numerical, float).
static bool find_best_threshold_numerical(const double* hist, const FeatureMeta& m, const Params& p, double sum_g,
                                          double sum_h, int32_t num_data, double parent, SplitInfo* out) {
  out->default_left = true;
  out->gain = K_MIN_SCORE;
  double sh = sum_h + 2.0 * EPS;
  Flags F{p.l1 > 0.0, p.max_delta > 0.0, p.smooth > EPS};
  double gain_shift = leaf_gain(F, sum_g, sh, p, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  bool sp = false;
  if (m.num_bin > 2 && m.missing != MISSING_NONE) {
    if (m.missing == MISSING_ZERO) {
      sp |= sequential(F, true, true, false, hist, m, p, sum_g, sh, num_data, mgs, parent, out);
      sp |= sequential(F, false, true, false, hist, m, p, sum_g, sh, num_data, mgs, parent, out);
    } else {
      sp |= sequential(F, true, false, true, hist, m, p, sum_g, sh, num_data, mgs, parent, out);
      sp |= sequential(F, false, false, true, hist, m, p, sum_g, sh, num_data, mgs, parent, out);
    }
  } else {
    sp |= sequential(F, true, false, false, hist, m, p, sum_g, sh, num_data, mgs, parent, out);
    if (m.missing == MISSING_NAN) out->default_left = false;
  }
  out->gain *= m.penalty;
  return sp;
}

// feature_histogram.rs:839-1142 — FindBestThresholdSequentiallyInt.
static bool sequential_int(const Flags& F, bool REV, bool SKIP, bool NA, const int64_t* hg, const int64_t* hh,
                           const FeatureMeta& m, const Params& p, int64_t tg, int64_t th, double gs, double hs,
                           int32_t num_data, double mgs, double parent, SplitInfo* out) {
  const int32_t offset = m.offset;
  bool is_splittable = false;
  int64_t best_lg = 0, best_lh = 0;
  double best_gain = K_MIN_SCORE;
  uint32_t best_th = (uint32_t)m.num_bin;
  double cnt_factor = (double)num_data / (double)th;
  auto gain_eps = [&](double slg, double slh, double srg, double srh, int32_t lc, int32_t rc) {
    double a = slh + EPS, b = srh + EPS;
    return gains(F, p, slg, a, srg, b, lc, rc, parent);
  };
  if (REV) {
    int64_t rg = 0, rh = 0;
    int t = m.num_bin - 1 - offset - (NA ? 1 : 0);
    int t_end = 1 - offset;
    for (; t >= t_end; --t) {
      if (SKIP && (t + offset) == m.default_bin) continue;
      rg += hg[t];
      rh += hh[t];
      int32_t rc = round_int((double)rh * cnt_factor);
      double srh = (double)rh * hs;
      if (rc < p.min_data || srh < p.min_hess) continue;
      int32_t lc = num_data - rc;
      if (lc < p.min_data) break;
      int64_t lh = th - rh;
      double slh = (double)lh * hs;
      if (slh < p.min_hess) break;
      int64_t lg = tg - rg;
      double slg = (double)lg * gs;
      double srg = (double)rg * gs;
      double cg = gain_eps(slg, slh, srg, srh, lc, rc);
      if (cg <= mgs) continue;
      is_splittable = true;
      if (cg > best_gain) {
        best_lg = lg;
        best_lh = lh;
        best_th = (uint32_t)(t - 1 + offset);
        best_gain = cg;
      }
    }
  } else {
    int64_t lg = 0, lh = 0;
    int t = 0;
    int t_end = m.num_bin - 2 - offset;
    if (NA && offset == 1) {
      lg = tg;
      lh = th;
      for (int i = 0; i < m.num_bin - offset; ++i) {
        lg -= hg[i];
        lh -= hh[i];
      }
      t = -1;
    }
    for (; t <= t_end; ++t) {
      if (SKIP && (t + offset) == m.default_bin) continue;
      if (t >= 0) {
        lg += hg[t];
        lh += hh[t];
      }
      int32_t lc = round_int((double)lh * cnt_factor);
      double slh = (double)lh * hs;
      if (lc < p.min_data || slh < p.min_hess) continue;
      int32_t rc = num_data - lc;
      if (rc < p.min_data) break;
      int64_t rh = th - lh;
      double srh = (double)rh * hs;
      if (srh < p.min_hess) break;
      int64_t rg = tg - lg;
      double slg = (double)lg * gs;
      double srg = (double)rg * gs;
      double cg = gain_eps(slg, slh, srg, srh, lc, rc);
      if (cg <= mgs) continue;
      is_splittable = true;
      if (cg > best_gain) {
        best_lg = lg;
        best_lh = lh;
        best_th = (uint32_t)(t + offset);
        best_gain = cg;
      }
    }
  }
  if (is_splittable && best_gain > out->gain + mgs) {
    int64_t rg = tg - best_lg, rh = th - best_lh;
    double slg = (double)best_lg * gs, slh = (double)best_lh * hs;
    double srg = (double)rg * gs, srh = (double)rh * hs;
    int32_t lc = round_int((double)best_lh * cnt_factor);
    int32_t rc = round_int((double)rh * cnt_factor);
    out->threshold = best_th;
    out->left_output = leaf_output(F, slg, slh, p, lc, parent);
    out->left_count = lc;
    out->lsg = slg;
    out->lsh = slh;
    out->right_output = leaf_output(F, srg, srh, p, rc, parent);
    out->right_count = rc;
    out->rsg = srg;
    out->rsh = srh;
    out->lint = (int64_t)(((uint64_t)best_lg << 32) | ((uint64_t)best_lh & 0xffffffffull));
    out->rint = (int64_t)(((uint64_t)rg << 32) | ((uint64_t)rh & 0xffffffffull));
    out->gain = best_gain - mgs;
    out->default_left = REV;
  }
  return is_splittable;
}

// feature_histogram.rs:673-830 — FindBestThresholdInt (numerical).
static bool find_best_threshold_numerical_int(const int64_t* hg, const int64_t* hh, const FeatureMeta& m,
                                              const Params& p, int64_t tg, int64_t th, double gs, double hs,
                                              int32_t num_data, double parent, SplitInfo* out) {
  out->default_left = true;
  out->gain = K_MIN_SCORE;
  double sg = (double)tg * gs;
  double sh = (double)th * hs;
  Flags F{p.l1 > 0.0, p.max_delta > 0.0, p.smooth > EPS};
  double gain_shift = leaf_gain(F, sg, sh, p, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  bool sp = false;
  if (m.num_bin > 2 && m.missing != MISSING_NONE) {
    if (m.missing == MISSING_ZERO) {
      sp |= sequential_int(F, true, true, false, hg, hh, m, p, tg, th, gs, hs, num_data, mgs, parent, out);
      sp |= sequential_int(F, false, true, false, hg, hh, m, p, tg, th, gs, hs, num_data, mgs, parent, out);
    } else {
      sp |= sequential_int(F, true, false, true, hg, hh, m, p, tg, th, gs, hs, num_data, mgs, parent, out);
      sp |= sequential_int(F, false, false, true, hg, hh, m, p, tg, th, gs, hs, num_data, mgs, parent, out);
    }
  } else {
    sp |= sequential_int(F, true, false, false, hg, hh, m, p, tg, th, gs, hs, num_data, mgs, parent, out);
    if (m.missing == MISSING_NAN) out->default_left = false;
  }
  out->gain *= m.penalty;
  return sp;
}

// ---------------------------------------------------------------------------------------------
// Categorical threshold search (feature_histogram.rs:1328-1886), no extra-trees draw, no
// monotone constraints: one-hot (one category against the rest) when num_bin <= max_cat_to_onehot,
// otherwise the categories with enough data sorted by grad / (hess + cat_smooth) and scanned from
// both ends for at most max_cat_threshold categories, with lambda_l2 + cat_l2.
// ---------------------------------------------------------------------------------------------

// min_gain_shift of a categorical search (feature_histogram.rs:1356-1386): with path smoothing
// the parent output is the leaf output, otherwise the unsmoothed leaf gain.
static double cat_gain_shift(const Flags& F, const Params& p, double sum_g, double sum_h, int32_t num_data,
                             double parent) {
  if (F.sm) return leaf_gain_given_output(F.l1, sum_g, sum_h, p, parent);
  Flags F0{F.l1, F.mx, false};
  return leaf_gain(F0, sum_g, sum_h, p, num_data, 0.0);
}

// The stable ascending order of `idx` by key (Rust's stable sort_by with partial_cmp).
static void stable_sort_by_key(std::vector<int32_t>& idx, const std::vector<double>& key) {
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return key[(size_t)a] < key[(size_t)b]; });
}

// Float form (feature_histogram.rs:1328-1598). hist: [g, h] per slice index.
static bool find_best_threshold_categorical(const double* hist, const FeatureMeta& m, const Params& p, double sum_g,
                                            double sum_h_in, int32_t num_data, double parent, SplitInfo* out) {
  const double sum_h = sum_h_in + 2.0 * EPS;
  out->default_left = false;
  out->gain = K_MIN_SCORE;
  Flags F{p.l1 > 0.0, p.max_delta > 0.0, p.smooth > EPS};
  const double mgs = cat_gain_shift(F, p, sum_g, sum_h, num_data, parent) + p.min_gain;
  const int32_t offset = m.offset, bin_start = 1 - offset, bin_end = m.num_bin - offset;
  auto grad = [&](int32_t t) { return hist[2 * t]; };
  auto hess = [&](int32_t t) { return hist[2 * t + 1]; };
  const double cnt_factor = (double)num_data / sum_h;
  const bool onehot = m.num_bin <= p.max_cat_to_onehot;
  Params pl = p;
  bool sp = false;
  double best_gain = K_MIN_SCORE, best_lg = 0.0, best_lh = 0.0;
  int32_t best_t = -1, best_dir = 1, best_lc = 0, used_bin = -1;
  std::vector<int32_t> sorted;
  if (onehot) {
    for (int32_t t = bin_start; t < bin_end; ++t) {
      const double g = grad(t), h = hess(t);
      const int32_t cnt = round_int(h * cnt_factor);
      if (cnt < p.min_data || h < p.min_hess) continue;
      const int32_t other_cnt = num_data - cnt;
      if (other_cnt < p.min_data) continue;
      const double other_h = sum_h - h - EPS;
      if (other_h < p.min_hess) continue;
      const double other_g = sum_g - g;
      const double gain = gains(F, pl, other_g, other_h, g, h + EPS, other_cnt, cnt, parent);
      if (!(gain > mgs)) continue;
      sp = true;
      if (gain > best_gain) {
        best_t = t;
        best_lg = g;
        best_lh = h + EPS;
        best_lc = cnt;
        best_gain = gain;
      }
    }
  } else {
    std::vector<double> key((size_t)std::max(bin_end, 0), 0.0);
    for (int32_t i = bin_start; i < bin_end; ++i) {
      if ((double)round_int(hess(i) * cnt_factor) >= p.cat_smooth) sorted.push_back(i);
      key[(size_t)i] = grad(i) / (hess(i) + p.cat_smooth);
    }
    used_bin = (int32_t)sorted.size();
    pl.l2 = p.l2 + p.cat_l2;
    stable_sort_by_key(sorted, key);
    const int32_t max_num_cat = std::min(p.max_cat_threshold, (used_bin + 1) / 2);
    for (int dir = 1, start = 0, pass = 0; pass < 2; ++pass, dir = -1, start = used_bin - 1) {
      int32_t pos = start, cnt_group = 0, left_cnt = 0;
      double lg = 0.0, lh = EPS;
      for (int32_t i = 0; i < used_bin && i < max_num_cat; ++i) {
        const int32_t t = sorted[(size_t)pos];
        pos += dir;
        const double g = grad(t), h = hess(t);
        const int32_t cnt = round_int(h * cnt_factor);
        lg += g;
        lh += h;
        left_cnt += cnt;
        cnt_group += cnt;
        if (left_cnt < p.min_data || lh < p.min_hess) continue;
        const int32_t right_cnt = num_data - left_cnt;
        if (right_cnt < p.min_data || right_cnt < p.min_data_per_group) break;
        const double rh = sum_h - lh;
        if (rh < p.min_hess) break;
        if (cnt_group < p.min_data_per_group) continue;
        cnt_group = 0;
        const double rg = sum_g - lg;
        const double gain = gains(F, pl, lg, lh, rg, rh, left_cnt, right_cnt, parent);
        if (gain > mgs) {
          sp = true;
          if (gain > best_gain) {
            best_lc = left_cnt;
            best_lg = lg;
            best_lh = lh;
            best_t = i;
            best_gain = gain;
            best_dir = dir;
          }
        }
      }
    }
  }
  if (sp) {
    out->left_output = leaf_output(F, best_lg, best_lh, pl, best_lc, parent);
    out->left_count = best_lc;
    out->lsg = best_lg;
    out->lsh = best_lh - EPS;
    out->right_output = leaf_output(F, sum_g - best_lg, sum_h - best_lh, pl, num_data - best_lc, parent);
    out->right_count = num_data - best_lc;
    out->rsg = sum_g - best_lg;
    out->rsh = sum_h - best_lh - EPS;
    out->gain = best_gain - mgs;
    out->cat_bins.clear();
    if (onehot) {
      out->cat_bins.push_back((uint32_t)(best_t + offset));
    } else {
      for (int32_t i = 0; i <= best_t; ++i) {
        const int32_t pos = best_dir == 1 ? i : used_bin - 1 - i;
        out->cat_bins.push_back((uint32_t)(sorted[(size_t)pos] + offset));
      }
    }
  }
  out->gain *= m.penalty;
  return sp;
}

// Integer form (feature_histogram.rs:1600-1886): exact integer sums scaled once; no kEpsilon.
static bool find_best_threshold_categorical_int(const int64_t* hg, const int64_t* hh, const FeatureMeta& m,
                                                const Params& p, int64_t tg, int64_t th, double gs, double hs,
                                                int32_t num_data, double parent, SplitInfo* out) {
  const double sum_g = (double)tg * gs, sum_h = (double)th * hs;
  out->default_left = false;
  out->gain = K_MIN_SCORE;
  Flags F{p.l1 > 0.0, p.max_delta > 0.0, p.smooth > EPS};
  const double mgs = cat_gain_shift(F, p, sum_g, sum_h, num_data, parent) + p.min_gain;
  const int32_t offset = m.offset, bin_start = 1 - offset, bin_end = m.num_bin - offset;
  const double cnt_factor = (double)num_data / (double)th;
  const bool onehot = m.num_bin <= p.max_cat_to_onehot;
  Params pl = p;
  bool sp = false;
  double best_gain = K_MIN_SCORE;
  int64_t best_ig = 0, best_ih = 0;
  int32_t best_t = -1, best_dir = 1, used_bin = -1;
  std::vector<int32_t> sorted;
  if (onehot) {
    for (int32_t t = bin_start; t < bin_end; ++t) {
      const int64_t ig = hg[t], ih = hh[t];
      const double h = (double)ih * hs;
      const int32_t cnt = round_int((double)ih * cnt_factor);
      if (cnt < p.min_data || h < p.min_hess) continue;
      const int32_t other_cnt = num_data - cnt;
      if (other_cnt < p.min_data) continue;
      const double other_h = (double)(th - ih) * hs;
      if (other_h < p.min_hess) continue;
      const double g = (double)ig * gs;
      const double other_g = (double)(tg - ig) * gs;
      const double gain = gains(F, pl, other_g, other_h, g, h, other_cnt, cnt, parent);
      if (!(gain > mgs)) continue;
      sp = true;
      if (gain > best_gain) {
        best_t = t;
        best_ig = ig;
        best_ih = ih;
        best_gain = gain;
      }
    }
  } else {
    std::vector<double> key((size_t)std::max(bin_end, 0), 0.0);
    for (int32_t i = bin_start; i < bin_end; ++i) {
      if ((double)round_int((double)hh[i] * cnt_factor) >= p.cat_smooth) sorted.push_back(i);
      key[(size_t)i] = ((double)hg[i] * gs) / ((double)hh[i] * hs + p.cat_smooth);
    }
    used_bin = (int32_t)sorted.size();
    pl.l2 = p.l2 + p.cat_l2;
    stable_sort_by_key(sorted, key);
    const int32_t max_num_cat = std::min(p.max_cat_threshold, (used_bin + 1) / 2);
    for (int dir = 1, start = 0, pass = 0; pass < 2; ++pass, dir = -1, start = used_bin - 1) {
      int32_t pos = start, cnt_group = 0, left_cnt = 0;
      int64_t lig = 0, lih = 0;
      for (int32_t i = 0; i < used_bin && i < max_num_cat; ++i) {
        const int32_t t = sorted[(size_t)pos];
        pos += dir;
        const int32_t cnt = round_int((double)hh[t] * cnt_factor);
        lig += hg[t];
        lih += hh[t];
        left_cnt += cnt;
        cnt_group += cnt;
        const double lh = (double)lih * hs;
        if (left_cnt < p.min_data || lh < p.min_hess) continue;
        const int32_t right_cnt = num_data - left_cnt;
        if (right_cnt < p.min_data || right_cnt < p.min_data_per_group) break;
        const double rh = (double)(th - lih) * hs;
        if (rh < p.min_hess) break;
        if (cnt_group < p.min_data_per_group) continue;
        cnt_group = 0;
        const double lg = (double)lig * gs, rg = (double)(tg - lig) * gs;
        const double gain = gains(F, pl, lg, lh, rg, rh, left_cnt, right_cnt, parent);
        if (gain > mgs) {
          sp = true;
          if (gain > best_gain) {
            best_ig = lig;
            best_ih = lih;
            best_t = i;
            best_gain = gain;
            best_dir = dir;
          }
        }
      }
    }
  }
  if (sp) {
    const double lg = (double)best_ig * gs, lh = (double)best_ih * hs;
    const int64_t rig = tg - best_ig, rih = th - best_ih;
    const double rg = (double)rig * gs, rh = (double)rih * hs;
    const int32_t lc = round_int((double)best_ih * cnt_factor), rc = round_int((double)rih * cnt_factor);
    out->left_output = leaf_output(F, lg, lh, pl, lc, parent);
    out->left_count = lc;
    out->lsg = lg;
    out->lsh = lh;
    out->right_output = leaf_output(F, rg, rh, pl, rc, parent);
    out->right_count = rc;
    out->rsg = rg;
    out->rsh = rh;
    out->lint = (int64_t)(((uint64_t)best_ig << 32) | ((uint64_t)best_ih & 0xffffffffULL));
    out->rint = (int64_t)(((uint64_t)rig << 32) | ((uint64_t)rih & 0xffffffffULL));
    out->gain = best_gain - mgs;
    out->cat_bins.clear();
    if (onehot) {
      out->cat_bins.push_back((uint32_t)(best_t + offset));
    } else {
      for (int32_t i = 0; i <= best_t; ++i) {
        const int32_t pos = best_dir == 1 ? i : used_bin - 1 - i;
        out->cat_bins.push_back((uint32_t)(sorted[(size_t)pos] + offset));
      }
    }
  }
  out->gain *= m.penalty;
  return sp;
}

// feature_histogram.rs:114-125 — leaf_output_root.
static double leaf_output_root(const Params& p, double sg, double sh, int32_t n) {
  Flags F{true, true, false};
  double r = leaf_output(F, sg, sh, p, n, 0.0);
  if (std::isnan(r)) return r;
  return std::min(std::max(r, -std::numeric_limits<double>::max()), std::numeric_limits<double>::max());
}

// ---------------------------------------------------------------------------------------------
// Partition routing (treelearner/data_partition.rs:299-410), single-feature dense group view:
// group_view (:25-40) gives min_bin = 1, max_bin = bin_offsets[1] - 1, use_min_bin = false.
// The rule is evaluated for every stored group bin into a route table (1 = left).
// ---------------------------------------------------------------------------------------------
static void route_table(const FeatureMeta& m, uint32_t threshold, bool default_left, int32_t group_bins,
                        uint8_t* lut) {
  const uint32_t min_bin = 1;
  const uint32_t max_bin = (uint32_t)group_bins - 1;
  const uint32_t default_bin = (uint32_t)m.default_bin;
  const uint32_t mfb = (uint32_t)m.mfb;
  bool miss_zero = false, miss_na = false, mfb_zero = false, mfb_na = false;
  if (m.missing == MISSING_ZERO) {
    miss_zero = true;
    mfb_zero = default_bin == mfb;
  } else if (m.missing == MISSING_NAN) {
    miss_na = true;
    mfb_na = (max_bin == mfb + 1) && mfb > 0;
  }
  uint32_t th = threshold + min_bin;
  uint32_t t_zero_bin = min_bin + default_bin;
  if (mfb == 0) {
    th -= 1;
    t_zero_bin -= 1;
  }
  const bool default_route_left = mfb <= threshold;
  const bool missing_default_left = (miss_zero || miss_na) && default_left;
  const bool max_bin_left = max_bin <= th;
  const bool multi_bin = min_bin < max_bin;
  for (int32_t b = 0; b < group_bins; ++b) {
    uint32_t bin = (uint32_t)b;
    bool left;
    if (multi_bin) {
      if ((miss_zero && !mfb_zero && bin == t_zero_bin) || (miss_na && !mfb_na && bin == max_bin)) {
        left = missing_default_left;
      } else if (bin == 0) {
        left = ((miss_na && mfb_na) || (miss_zero && mfb_zero)) ? missing_default_left : default_route_left;
      } else {
        left = !(bin > th);
      }
    } else if (miss_zero && !mfb_zero && bin == t_zero_bin) {
      left = missing_default_left;
    } else if (bin != max_bin) {
      left = ((miss_na && mfb_na) || (miss_zero && mfb_zero)) ? missing_default_left : default_route_left;
    } else if (miss_na && !mfb_na) {
      left = missing_default_left;
    } else {
      left = max_bin_left;
    }
    lut[b] = left ? 1 : 0;
  }
}

// Categorical routing (data_partition.rs:264-300, route_bin :367-377): group bin 0 (the most
// frequent bin's rows) takes the default route — left when the most frequent bin is in the bitset
// and not 0 —, any other stored bin b looks up bit b - 1 + offset of the bin bitset.
static void route_table_cat(const FeatureMeta& m, const uint32_t* bits, int32_t group_bins, uint8_t* lut) {
  const uint32_t mfb = (uint32_t)m.mfb, offset = m.mfb == 0 ? 1u : 0u;
  auto in_bits = [&](uint32_t pos) { return pos < 256 && ((bits[pos / 32] >> (pos % 32)) & 1u) != 0; };
  const bool default_left = mfb > 0 && in_bits(mfb);
  for (int32_t b = 0; b < group_bins; ++b) lut[b] = b == 0 ? (default_left ? 1 : 0) : (in_bits((uint32_t)b - 1 + offset) ? 1 : 0);
}

// utils/random.rs:6-80 — LightGBM's LCG and its k-of-n sample, for the by-node column sample.
struct Lcg {
  uint32_t x = 0;
  uint32_t step() {
    x = x * 214013u + 2531011u;
    return x;
  }
  int32_t next_int(int32_t lo, int32_t hi) { return (int32_t)(step() & 0x7fffffffu) % (hi - lo) + lo; }
  float next_float() { return (float)((step() >> 16) & 0x7fffu) / 32768.0f; }
  std::vector<int32_t> sample(int32_t n, int32_t k) {
    std::vector<int32_t> ret;
    if (k > n || k <= 0) return ret;
    if (k == n) {
      for (int32_t i = 0; i < n; ++i) ret.push_back(i);
      return ret;
    }
    if (k > 1 && (double)k > (double)n / std::log2((double)k)) {
      for (int32_t i = 0; i < n; ++i) {
        const double prob = (double)(k - (int32_t)ret.size()) / (double)(n - i);
        if ((double)next_float() < prob) ret.push_back(i);
      }
      return ret;
    }
    std::vector<uint8_t> in((size_t)n, 0);
    for (int32_t r = n - k; r < n; ++r) {
      const int32_t v = next_int(0, r + 1);
      if (in[(size_t)v]) in[(size_t)r] = 1;
      else in[(size_t)v] = 1;
    }
    for (int32_t i = 0; i < n; ++i)
      if (in[(size_t)i]) ret.push_back(i);
    return ret;
  }
};

// col_sampler.rs:14-20 — GetCnt.
static int32_t col_get_cnt(int32_t total, double fraction) {
  const int32_t mn = std::min(1, total);
  const int32_t used = (int32_t)((double)total * fraction + 0.5);
  return std::max(used, mn);
}

static void bitset_of(const std::vector<uint32_t>& vals, uint32_t* bits) {
  for (int i = 0; i < 8; ++i) bits[i] = 0;
  for (uint32_t v : vals)
    if (v < 256) bits[v / 32] |= 1u << (v % 32);
}

// ---------------------------------------------------------------------------------------------
// A persistent worker pool: the reference runs its per-feature histogram and search tasks on
// rayon (serial.rs:1022-1038, :1481-1489). Every task owns its feature's slices and the results
// are folded in feature order afterwards, so any thread count gives the same tree.
// ---------------------------------------------------------------------------------------------
struct Pool {
  std::vector<std::thread> workers;
  std::mutex m;
  std::condition_variable cv, done_cv;
  std::function<void(int)> job;
  int njobs = 0, active = 0;
  std::atomic<int> next{0};
  uint64_t gen = 0;
  bool quit = false;

  explicit Pool(int threads) {
    for (int t = 1; t < threads; ++t) workers.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m);
      quit = true;
    }
    cv.notify_all();
    for (auto& w : workers) w.join();
  }
  void work() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= njobs) break;
      job(i);
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return quit || gen != seen; });
        if (quit) return;
        seen = gen;
      }
      work();
      {
        std::lock_guard<std::mutex> g(m);
        if (--active == 0) done_cv.notify_all();
      }
    }
  }
  void run(int n, const std::function<void(int)>& f) {
    if (workers.empty() || n < 2) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m);
      job = f;
      njobs = n;
      next = 0;
      active = (int)workers.size();
      ++gen;
    }
    cv.notify_all();
    work();
    std::unique_lock<std::mutex> lk(m);
    done_cv.wait(lk, [&] { return active == 0; });
  }
};

// ---------------------------------------------------------------------------------------------
// Learner (treelearner/serial.rs)
// ---------------------------------------------------------------------------------------------
struct SplitRecord {  // one split: the arguments of tree.split_numerical / split_categorical
  int32_t leaf, right_leaf, inner_feature, real_feature;
  uint32_t threshold;
  int32_t default_left, missing_type, left_count, right_count;
  double left_output, right_output, left_sum_gradient, left_sum_hessian, right_sum_gradient, right_sum_hessian,
      gain;
  int64_t left_int_sum, right_int_sum;
  int32_t categorical, _pad;
  uint32_t cat_bins[8];  // categorical: bitset of the bins that go left (construct_bitset, utils/common.rs:221)
};

struct LeafSplits {  // serial.rs:53-76
  int32_t leaf = -1, num_data = 0;
  double sg = 0, sh = 0, weight = 0;
  int64_t int_sum = 0;
};

struct Learner {
  // dataset
  int64_t n = 0;
  int32_t nf = 0;
  std::vector<FeatureMeta> metas;
  std::vector<const uint8_t*> cols;  // stored group bins per inner feature
  std::vector<int64_t> gstart;       // first group bin of each feature in a slot
  std::vector<int32_t> gbins;        // group bins of each feature
  int64_t total_bins = 0;
  // config
  Params p;
  int32_t num_leaves = 31, max_depth = -1;
  bool const_hess = false, quant = false, renew_leaf = false, stoch = false;
  int32_t quant_bins = 4;
  // state
  std::vector<std::vector<double>> slots;
  std::vector<std::vector<int64_t>> islots_g, islots_h;
  std::vector<std::vector<uint8_t>> splittable;
  std::vector<int32_t> leaf_slot;
  int32_t next_free = 0;
  std::vector<int64_t> leaf_begin, leaf_count;
  std::vector<int32_t> indices;
  std::vector<SplitInfo> best;
  std::vector<int32_t> leaf_depth;
  Discretizer disc;
  double gscale = 0, hscale = 0;
  LeafSplits smaller, larger;
  int32_t smaller_slot = 0, larger_slot = -1, parent_slot = -1;
  std::vector<SplitRecord> records;
  std::vector<double> leaf_value;
  // the features of each leaf's last search (its histogram slot holds their histograms; the
  // slot's other features are left from earlier use)
  std::vector<std::vector<uint8_t>> leaf_used;
  int32_t tree_leaves = 1;
  double root_output = 0.0;
  std::vector<float> og, oh;
  std::vector<uint8_t> tree_mask;  // empty: every feature is used by the tree
  // by-node column sample (col_sampler.rs:109-177 without interaction constraints)
  double bynode_fraction = 1.0;
  bool bytree_active = false;
  Lcg node_rng;

  // interaction constraints (config interaction_constraints, col_sampler.rs:148-177): sets of inner
  // features; the features on the path to each leaf (serial.rs:233-234, :1719-1722)
  std::vector<std::vector<uint8_t>> icons;
  std::vector<std::vector<uint8_t>> branch;

  // ColSampler::allowed_features: the path's features, plus every constraint that contains the
  // whole path (every constraint at the root)
  std::vector<uint8_t> allowed_features(int32_t leaf) {
    const std::vector<uint8_t>& b = branch[(size_t)leaf];
    std::vector<uint8_t> allowed = b;
    bool empty = true;
    for (uint8_t x : b) empty = empty && !x;
    for (const auto& c : icons) {
      bool all = true;
      for (int32_t f = 0; f < nf; ++f) all = all && (!b[(size_t)f] || c[(size_t)f]);
      if (empty || all)
        for (int32_t f = 0; f < nf; ++f) allowed[(size_t)f] |= c[(size_t)f];
    }
    return allowed;
  }

  // ColSampler::get_by_node: the features a searched leaf may split on
  std::vector<uint8_t> node_mask(int32_t leaf) {
    std::vector<uint8_t> ret((size_t)nf, 0);
    const bool constrained = !icons.empty();
    const std::vector<uint8_t> allowed = constrained ? allowed_features(leaf) : std::vector<uint8_t>();
    if (bynode_fraction >= 1.0) {
      if (!constrained) {
        std::fill(ret.begin(), ret.end(), 1);
        return ret;
      }
      return allowed;
    }
    std::vector<int32_t> cand;  // the by-tree sample or every feature, ascending
    for (int32_t f = 0; f < nf; ++f)
      if (!bytree_active || tree_mask.empty() || tree_mask[(size_t)f]) cand.push_back(f);
    int32_t cnt = col_get_cnt((int32_t)cand.size(), bynode_fraction);
    if (constrained) {
      std::vector<int32_t> filtered;
      for (int32_t f : cand)
        if (allowed[(size_t)f]) filtered.push_back(f);
      cand.swap(filtered);
      cnt = std::min(cnt, (int32_t)cand.size());
    }
    for (int32_t q : node_rng.sample((int32_t)cand.size(), cnt)) ret[(size_t)cand[(size_t)q]] = 1;
    return ret;
  }
  Pool* workers = nullptr;
  ~Learner() { delete workers; }

  int32_t pool_get(int32_t leaf, bool* had) {  // serial.rs:117-141 (full pool)
    if (leaf_slot[leaf] >= 0) {
      *had = true;
      return leaf_slot[leaf];
    }
    *had = false;
    int32_t s = next_free++;
    leaf_slot[leaf] = s;
    return s;
  }
  void pool_move(int32_t src, int32_t dst) {  // serial.rs:151-161
    int32_t s = leaf_slot[src];
    if (s >= 0) {
      leaf_slot[src] = -1;
      leaf_slot[dst] = s;
    }
  }

  void setup() {
    gstart.resize(nf);
    gbins.resize(nf);
    int64_t cur = 0;
    for (int f = 0; f < nf; ++f) {
      gstart[f] = cur;
      gbins[f] = 1 + metas[f].num_bin - metas[f].offset;
      cur += gbins[f];
    }
    total_bins = cur;
    slots.assign(num_leaves, std::vector<double>(2 * total_bins, 0.0));
    if (quant) {
      islots_g.assign(num_leaves, std::vector<int64_t>(total_bins, 0));
      islots_h.assign(num_leaves, std::vector<int64_t>(total_bins, 0));
    }
    splittable.assign(num_leaves, std::vector<uint8_t>(nf, 1));
    leaf_slot.assign(num_leaves, -1);
    leaf_begin.assign(num_leaves, 0);
    leaf_count.assign(num_leaves, 0);
    indices.resize(n);
    best.assign(num_leaves, SplitInfo());
    leaf_depth.assign(num_leaves, 0);
    leaf_value.assign(num_leaves, 0.0);
    leaf_used.assign(num_leaves, std::vector<uint8_t>(nf, 0));
  }

  const int32_t* leaf_rows(int32_t leaf) const { return indices.data() + leaf_begin[leaf]; }

  // serial.rs:891-1065 — float histograms of one leaf into `slot` (dense single-value groups).
  void construct_histograms(const std::vector<uint8_t>& used, int32_t leaf, int32_t slot, const float* g,
                            const float* h) {
    int64_t cnt = leaf_count[leaf];
    const int32_t* ix = cnt < n ? leaf_rows(leaf) : nullptr;
    const float* pg = g;
    const float* ph = h;
    if (ix) {
      og.resize(cnt);
      for (int64_t i = 0; i < cnt; ++i) og[i] = g[ix[i]];
      if (!const_hess) {
        oh.resize(cnt);
        for (int64_t i = 0; i < cnt; ++i) oh[i] = h[ix[i]];
      }
      pg = og.data();
      ph = const_hess ? h : oh.data();
    }
    std::vector<double>& hist = slots[slot];
    workers->run(nf, [&](int f) {
      if (!used[f]) return;
      double* out = hist.data() + 2 * gstart[f];
      std::fill(out, out + 2 * gbins[f], 0.0);
      const uint8_t* col = cols[f];
      for (int64_t i = 0; i < cnt; ++i) {
        int64_t row = ix ? ix[i] : i;
        size_t ti = (size_t)col[row] << 1;
        out[ti] += (double)pg[i];
        out[ti + 1] += const_hess ? 1.0 : (double)ph[i];
      }
      if (const_hess) {
        double h0 = (double)h[0];
        for (int b = 0; b < gbins[f]; ++b) out[2 * b + 1] *= h0;
      }
    });
  }

  // serial.rs:1074-1164 — integer histograms of one leaf.
  void construct_int_histograms(const std::vector<uint8_t>& used, int32_t leaf, int32_t slot) {
    int64_t cnt = leaf_count[leaf];
    const int32_t* ix = cnt < n ? leaf_rows(leaf) : nullptr;
    const int16_t* pk = disc.packed.data();
    workers->run(nf, [&](int f) {
      if (!used[f]) return;
      int64_t* og_ = islots_g[slot].data() + gstart[f];
      int64_t* oh_ = islots_h[slot].data() + gstart[f];
      std::fill(og_, og_ + gbins[f], 0);
      std::fill(oh_, oh_ + gbins[f], 0);
      const uint8_t* col = cols[f];
      for (int64_t i = 0; i < cnt; ++i) {
        int64_t row = ix ? ix[i] : i;
        int16_t pv = pk[row];
        int b = col[row];
        og_[b] += (int64_t)(int8_t)(pv >> 8);
        oh_[b] += (int64_t)(uint8_t)(pv & 0xff);
      }
    });
  }

  // serial.rs:2205-2238 — FixHistogram on one feature slice (feature-local bins).
  static void fix_slice(double* d, int mfb, int num_bin, double sg, double sh) {
    if (mfb > 0) {
      d[mfb << 1] = sg;
      d[(mfb << 1) + 1] = sh;
      for (int i = 0; i < num_bin; ++i) {
        if (i != mfb) {
          d[mfb << 1] -= d[i << 1];
          d[(mfb << 1) + 1] -= d[(i << 1) + 1];
        }
      }
    }
  }
  static void fix_slice_int(int64_t* dg, int64_t* dh, int mfb, int num_bin, int64_t tg, int64_t th) {
    if (mfb > 0) {
      dg[mfb] = tg;
      dh[mfb] = th;
      for (int i = 0; i < num_bin; ++i) {
        if (i != mfb) {
          dg[mfb] -= dg[i];
          dh[mfb] -= dh[i];
        }
      }
    }
  }

  // serial.rs:1322-1566 (sequential phases) and :1212-1300 (integer phases).
  void find_best_splits_from_histograms(const std::vector<uint8_t>& used, bool use_subtract, double sp_out,
                                        double lp_out) {
    int32_t lslot = larger.leaf >= 0 ? larger_slot : -1;
    // serial.rs:1328-1336 — the by-node samples of the smaller leaf, then the larger one
    const std::vector<uint8_t> smask = node_mask(smaller.leaf);
    const std::vector<uint8_t> lmask =
        larger.leaf >= 0 ? node_mask(larger.leaf) : std::vector<uint8_t>((size_t)nf, 1);
    std::vector<SplitInfo> cs_all(nf), cl_all(nf);
    std::vector<uint8_t> ss_all(nf, 0), sl_all(nf, 0);
    workers->run(nf, [&](int f) {
      if (!used[f]) return;
      const FeatureMeta& m = metas[f];
      int64_t start = gstart[f] + 1;  // feature_hist_offsets: group start + bin_offsets[0]
      int len = m.num_bin - m.offset;
      SplitInfo cs, cl;
      bool ss, sl = false;
      if (quant) {
        int64_t* sg_ = islots_g[smaller_slot].data() + start;
        int64_t* sh_ = islots_h[smaller_slot].data() + start;
        fix_slice_int(sg_, sh_, m.mfb, m.num_bin, smaller.int_sum >> 32, smaller.int_sum & 0xffffffffLL);
        if (lslot >= 0) {
          int64_t* lg_ = islots_g[lslot].data() + start;
          int64_t* lh_ = islots_h[lslot].data() + start;
          if (use_subtract) {
            for (int i = 0; i < len; ++i) {
              lg_[i] -= sg_[i];
              lh_[i] -= sh_[i];
            }
          } else {
            fix_slice_int(lg_, lh_, m.mfb, m.num_bin, larger.int_sum >> 32, larger.int_sum & 0xffffffffLL);
          }
        }
        // serial.rs:2381-2433 — categorical features take the categorical search
        auto search_int = m.categorical ? find_best_threshold_categorical_int : find_best_threshold_numerical_int;
        ss = search_int(sg_, sh_, m, p, smaller.int_sum >> 32, smaller.int_sum & 0xffffffffLL, gscale, hscale,
                        smaller.num_data, sp_out, &cs);
        if (lslot >= 0) {
          int64_t* lg_ = islots_g[lslot].data() + start;
          int64_t* lh_ = islots_h[lslot].data() + start;
          sl = search_int(lg_, lh_, m, p, larger.int_sum >> 32, larger.int_sum & 0xffffffffLL, gscale, hscale,
                          larger.num_data, lp_out, &cl);
        }
      } else {
        double* sd = slots[smaller_slot].data() + 2 * start;
        fix_slice(sd, m.mfb, m.num_bin, smaller.sg, smaller.sh);
        if (lslot >= 0) {
          double* ld = slots[lslot].data() + 2 * start;
          if (use_subtract) {
            for (int i = 0; i < 2 * len; ++i) ld[i] -= sd[i];
          } else {
            fix_slice(ld, m.mfb, m.num_bin, larger.sg, larger.sh);
          }
        }
        // serial.rs:2335-2379
        auto search = m.categorical ? find_best_threshold_categorical : find_best_threshold_numerical;
        ss = search(sd, m, p, smaller.sg, smaller.sh, smaller.num_data, sp_out, &cs);
        if (lslot >= 0) {
          double* ld = slots[lslot].data() + 2 * start;
          sl = search(ld, m, p, larger.sg, larger.sh, larger.num_data, lp_out, &cl);
        }
      }
      cs.feature = m.real;
      cl.feature = m.real;
      cs_all[f] = cs;
      cl_all[f] = cl;
      ss_all[f] = ss;
      sl_all[f] = sl;
    });
    // serial.rs:1523-1558 — fold in feature order
    SplitInfo sbest, lbest;
    for (int f = 0; f < nf; ++f) {
      if (!used[f]) continue;
      splittable[smaller_slot][f] = ss_all[f];
      if (smask[(size_t)f] && cs_all[f].better_than(sbest)) sbest = cs_all[f];
      if (lslot >= 0) {
        splittable[lslot][f] = sl_all[f];
        if (lmask[(size_t)f] && cl_all[f].better_than(lbest)) lbest = cl_all[f];
      }
    }
    best[smaller.leaf] = sbest;
    if (larger.leaf >= 0) best[larger.leaf] = lbest;
    leaf_used[(size_t)smaller.leaf] = used;
    if (larger.leaf >= 0) leaf_used[(size_t)larger.leaf] = used;
  }

  // serial.rs:779-825
  bool before_find_best_split(int32_t left, int32_t right) {
    if (max_depth > 0 && leaf_depth[left] >= max_depth) {
      best[left].gain = K_MIN_SCORE;
      if (right >= 0) best[right].gain = K_MIN_SCORE;
      return false;
    }
    int32_t nl = (int32_t)leaf_count[left];
    int32_t nr = right >= 0 ? (int32_t)leaf_count[right] : 0;
    if (nr < p.min_data * 2 && nl < p.min_data * 2) {
      best[left].gain = K_MIN_SCORE;
      if (right >= 0) best[right].gain = K_MIN_SCORE;
      return false;
    }
    parent_slot = -1;
    bool had;
    if (right < 0) {
      smaller_slot = pool_get(left, &had);
      larger_slot = -1;
    } else if (nl < nr) {
      int32_t ls = pool_get(left, &had);
      if (had) parent_slot = ls;
      larger_slot = ls;
      pool_move(left, right);
      smaller_slot = pool_get(left, &had);
    } else {
      int32_t ls = pool_get(left, &had);
      if (had) parent_slot = ls;
      larger_slot = ls;
      smaller_slot = pool_get(right, &had);
    }
    return true;
  }

  // serial.rs:830-887; the by-tree feature mask (ColSampler::is_feature_used_bytree,
  // col_sampler.rs:87-108) skips a feature before the splittable propagation (serial.rs:841-846)
  void find_best_splits(const float* g, const float* h) {
    std::vector<uint8_t> used(nf, 0);
    for (int f = 0; f < nf; ++f) {
      if (!tree_mask.empty() && !tree_mask[f]) continue;
      if (parent_slot >= 0 && !splittable[parent_slot][f]) {
        splittable[smaller_slot][f] = 0;
        continue;
      }
      used[f] = 1;
    }
    bool use_subtract = parent_slot >= 0;
    if (quant) construct_int_histograms(used, smaller.leaf, smaller_slot);
    else construct_histograms(used, smaller.leaf, smaller_slot, g, h);
    if (larger_slot >= 0 && !use_subtract && larger.leaf >= 0) {
      if (quant) construct_int_histograms(used, larger.leaf, larger_slot);
      else construct_histograms(used, larger.leaf, larger_slot, g, h);
    }
    // serial.rs:1924-1935 — parent output is the root output at the root, else the leaf weight.
    double sp_out = tree_leaves == 1 ? leaf_output_root(p, smaller.sg, smaller.sh, smaller.num_data) : smaller.weight;
    double lp_out = 0.0;
    if (larger.leaf >= 0)
      lp_out = tree_leaves == 1 ? leaf_output_root(p, larger.sg, larger.sh, larger.num_data) : larger.weight;
    find_best_splits_from_histograms(used, use_subtract, sp_out, lp_out);
  }

  // data_partition.rs:124-174 — stable split of `leaf` into itself (left) and `right_leaf`.
  void partition_split(int32_t leaf, int32_t right_leaf, int32_t f, uint32_t threshold, bool default_left,
                       const uint32_t* cat_bits) {
    uint8_t lut[65536];
    if (cat_bits) route_table_cat(metas[f], cat_bits, gbins[f], lut);
    else route_table(metas[f], threshold, default_left, gbins[f], lut);
    int64_t b = leaf_begin[leaf], c = leaf_count[leaf];
    const uint8_t* col = cols[f];
    // data_partition.rs:137-159 — a leaf of at least 2048 rows is routed in one contiguous block
    // of rows per thread; each block keeps its rows' order and the blocks are concatenated in
    // order, which is the sequential stable partition
    const int64_t threads = workers ? (int64_t)workers->workers.size() + 1 : 1;
    const int64_t block_len = (threads > 1 && c >= 2048) ? (c + threads - 1) / threads : std::max<int64_t>(c, 1);
    const int64_t blocks = (c + block_len - 1) / block_len;
    std::vector<std::vector<int32_t>> L((size_t)std::max<int64_t>(blocks, 1)), R(L.size());
    auto route_block = [&](int k) {
      const int64_t lo = (int64_t)k * block_len, hi = std::min(c, lo + block_len);
      L[(size_t)k].reserve((size_t)(hi - lo));
      R[(size_t)k].reserve((size_t)(hi - lo));
      for (int64_t i = lo; i < hi; ++i) {
        int32_t r = indices[b + i];
        if (lut[col[r]]) L[(size_t)k].push_back(r);
        else R[(size_t)k].push_back(r);
      }
    };
    if (blocks > 1) workers->run((int)blocks, route_block);
    else if (blocks == 1) route_block(0);
    int64_t pos = b;
    for (const auto& v : L) {
      std::copy(v.begin(), v.end(), indices.begin() + pos);
      pos += (int64_t)v.size();
    }
    const int64_t left = pos - b;
    for (const auto& v : R) {
      std::copy(v.begin(), v.end(), indices.begin() + pos);
      pos += (int64_t)v.size();
    }
    leaf_count[leaf] = left;
    leaf_begin[right_leaf] = b + left;
    leaf_count[right_leaf] = c - left;
  }

  static double round_to_zero(double v) {  // tree.rs:66-68,299-301
    return (v >= -K_ZERO_THRESHOLD && v <= K_ZERO_THRESHOLD) ? 0.0 : v;
  }

  // serial.rs:1685-1876 (numerical split, no constraints).
  void split(int32_t best_leaf, int32_t* out_left, int32_t* out_right) {
    SplitInfo info = best[best_leaf];
    int32_t inner = -1;
    for (int f = 0; f < nf; ++f)
      if (metas[f].real == info.feature) inner = f;
    int32_t next_leaf = tree_leaves;
    // serial.rs:1724-1745 — a categorical split partitions by the bitset of its bins
    // serial.rs:1719-1722 — both children's paths gain the split feature
    branch[(size_t)next_leaf] = branch[(size_t)best_leaf];
    branch[(size_t)next_leaf][(size_t)inner] = 1;
    branch[(size_t)best_leaf][(size_t)inner] = 1;
    const bool cat = metas[inner].categorical != 0;
    uint32_t bits[8];
    bitset_of(info.cat_bins, bits);
    partition_split(best_leaf, next_leaf, inner, info.threshold, info.default_left, cat ? bits : nullptr);
    info.left_count = (int32_t)leaf_count[best_leaf];
    info.right_count = (int32_t)leaf_count[next_leaf];
    SplitRecord r;
    std::memset(&r, 0, sizeof(r));
    r.categorical = cat ? 1 : 0;
    for (int i = 0; i < 8; ++i) r.cat_bins[i] = cat ? bits[i] : 0u;
    r.leaf = best_leaf;
    r.right_leaf = next_leaf;
    r.inner_feature = inner;
    r.real_feature = info.feature;
    r.threshold = cat ? 0u : info.threshold;
    r.default_left = info.default_left ? 1 : 0;
    r.missing_type = metas[inner].missing;
    r.left_count = info.left_count;
    r.right_count = info.right_count;
    r.left_output = info.left_output;
    r.right_output = info.right_output;
    r.left_sum_gradient = info.lsg;
    r.left_sum_hessian = info.lsh;
    r.right_sum_gradient = info.rsg;
    r.right_sum_hessian = info.rsh;
    r.gain = info.gain;
    r.left_int_sum = info.lint;
    r.right_int_sum = info.rint;
    records.push_back(r);
    // tree.rs:344-353 — leaf values of the children
    leaf_value[best_leaf] = std::isnan(info.left_output) ? 0.0 : info.left_output;
    leaf_value[next_leaf] = std::isnan(info.right_output) ? 0.0 : info.right_output;
    tree_leaves += 1;
    leaf_depth[next_leaf] = leaf_depth[best_leaf] + 1;
    leaf_depth[best_leaf] += 1;
    LeafSplits l{best_leaf, info.left_count, info.lsg, info.lsh, info.left_output, info.lint};
    LeafSplits rr{next_leaf, info.right_count, info.rsg, info.rsh, info.right_output, info.rint};
    if (info.left_count < info.right_count) {
      smaller = l;
      larger = rr;
    } else {
      smaller = rr;
      larger = l;
    }
    best[best_leaf] = info;
    *out_left = best_leaf;
    *out_right = next_leaf;
  }

  // serial.rs:658-776 (no bagging / column sampling / constraints)
  void before_train(const float* g, const float* h, const int32_t* rows, int64_t nrows) {
    for (auto& u : leaf_used) std::fill(u.begin(), u.end(), 0);
    std::fill(leaf_slot.begin(), leaf_slot.end(), -1);
    next_free = 0;
    std::fill(leaf_depth.begin(), leaf_depth.end(), 0);
    std::fill(leaf_begin.begin(), leaf_begin.end(), 0);
    std::fill(leaf_count.begin(), leaf_count.end(), 0);
    if (rows) {
      leaf_count[0] = nrows;
      std::copy(rows, rows + nrows, indices.begin());
    } else {
      leaf_count[0] = n;
      for (int64_t i = 0; i < n; ++i) indices[i] = (int32_t)i;
    }
    for (auto& s : best) {
      s.feature = -1;
      s.gain = K_MIN_SCORE;
    }
    if (quant) {
      bool ok = stoch ? disc.discretize_stochastic(g, h) : disc.discretize_nearest(g, h);
      if (ok) {
        gscale = disc.gscale;
        hscale = disc.hscale;
      }
    }
    double sg = 0, sh = 0;
    int64_t isum = 0;
    int64_t count = rows ? nrows : n;
    for (int64_t k = 0; k < count; ++k) {
      int64_t i = rows ? rows[k] : k;
      if (quant) {
        int16_t pv = disc.packed[i];
        int8_t gi = (int8_t)(pv >> 8);
        uint8_t hi = (uint8_t)(pv & 0xff);
        sg += (double)gi * gscale;
        sh += (double)hi * hscale;
        isum += (int64_t)(((uint64_t)(int64_t)gi << 32) | (uint64_t)hi);
      } else {
        sg += (double)g[i];
        sh += (double)h[i];
      }
    }
    double carried = smaller.weight;
    smaller = LeafSplits{0, (int32_t)count, sg, sh, carried, isum};
    larger = LeafSplits();
  }

  // serial.rs:634-655
  void renew_outputs(const float* g, const float* h) {
    Flags F{true, true, false};
    for (int32_t leaf = 0; leaf < tree_leaves; ++leaf) {
      const int32_t* ix = leaf_rows(leaf);
      int64_t c = leaf_count[leaf];
      double s1 = 0, s2 = 0;
      for (int64_t k = 0; k < c; ++k) {
        s1 += (double)g[ix[k]];
        s2 += (double)h[ix[k]];
      }
      double o = leaf_output(F, s1, s2, p, (int32_t)c, 0.0);
      leaf_value[leaf] = round_to_zero(o);
    }
  }

  // serial.rs:578-628
  void train(const float* g, const float* h, const int32_t* rows, int64_t nrows) {
    branch.assign((size_t)num_leaves, std::vector<uint8_t>((size_t)nf, 0));  // serial.rs:660-662
    before_train(g, h, rows, nrows);
    records.clear();
    std::fill(leaf_value.begin(), leaf_value.end(), 0.0);
    tree_leaves = 1;
    double root = leaf_output_root(p, smaller.sg, smaller.sh, smaller.num_data);
    leaf_value[0] = round_to_zero(root);
    root_output = leaf_value[0];
    int32_t left = 0, right = -1;
    for (int32_t it = 0; it < num_leaves - 1; ++it) {
      if (before_find_best_split(left, right)) find_best_splits(g, h);
      int32_t bl = 0;
      for (int32_t i = 1; i < num_leaves; ++i)
        if (best[i].better_than(best[bl])) bl = i;
      if (best[bl].gain <= 0.0) break;
      split(bl, &left, &right);
    }
    if (quant && renew_leaf) renew_outputs(g, h);
  }
};

}  // namespace orc

// ---------------------------------------------------------------------------------------------
// C entry points for the Python test harness (ctypes).
// ---------------------------------------------------------------------------------------------
using namespace orc;

extern "C" {

typedef struct {
  int32_t num_bin, missing_type, default_bin, most_freq_bin;
  double penalty;
  int32_t real_feature, bin_type;  // bin_type: 0 numerical, 1 categorical
} orc_feature;

typedef struct {
  int32_t num_leaves, max_depth, min_data_in_leaf, _pad0;
  double min_sum_hessian_in_leaf, lambda_l1, lambda_l2, max_delta_step, path_smooth, min_gain_to_split;
  int32_t use_quantized_grad, num_grad_quant_bins, quant_train_renew_leaf, stochastic_rounding;
  int32_t seed, num_threads, fused_madd, is_constant_hessian;
  int32_t max_cat_to_onehot, max_cat_threshold;
  double cat_smooth, cat_l2;
  int32_t min_data_per_group, _pad1;
} orc_config;

typedef SplitRecord orc_split;

void* orc_learner_create(const orc_feature* feats, int32_t nf, const uint8_t* bins_colmajor, int64_t n,
                         const orc_config* c) {
  Learner* L = new Learner();
  L->n = n;
  L->nf = nf;
  for (int f = 0; f < nf; ++f) {
    FeatureMeta m;
    m.num_bin = feats[f].num_bin;
    m.missing = feats[f].missing_type;
    m.default_bin = feats[f].default_bin;
    m.mfb = feats[f].most_freq_bin;
    m.offset = m.mfb == 0 ? 1 : 0;
    m.penalty = feats[f].penalty;
    m.real = feats[f].real_feature;
    m.categorical = feats[f].bin_type == 1 ? 1 : 0;
    L->metas.push_back(m);
    L->cols.push_back(bins_colmajor + (size_t)f * (size_t)n);
  }
  L->p.l1 = c->lambda_l1;
  L->p.l2 = c->lambda_l2;
  L->p.max_delta = c->max_delta_step;
  L->p.smooth = c->path_smooth;
  L->p.min_data = c->min_data_in_leaf;
  L->p.min_hess = c->min_sum_hessian_in_leaf;
  L->p.min_gain = c->min_gain_to_split;
  L->p.fused = c->fused_madd != 0;
  L->p.max_cat_to_onehot = c->max_cat_to_onehot;
  L->p.max_cat_threshold = c->max_cat_threshold;
  L->p.cat_smooth = c->cat_smooth;
  L->p.cat_l2 = c->cat_l2;
  L->p.min_data_per_group = c->min_data_per_group;
  L->num_leaves = c->num_leaves;
  L->max_depth = c->max_depth;
  L->const_hess = c->is_constant_hessian != 0;
  L->quant = c->use_quantized_grad != 0 && c->num_grad_quant_bins >= 2 && c->num_grad_quant_bins <= 127;
  L->quant_bins = c->num_grad_quant_bins;
  L->renew_leaf = c->quant_train_renew_leaf != 0;
  L->stoch = c->stochastic_rounding != 0;
  L->setup();
  L->workers = new Pool(c->num_threads > 0 ? c->num_threads : 1);
  if (L->quant) {
    L->disc.init((size_t)n, c->num_grad_quant_bins, L->const_hess, L->p.fused);
    if (L->stoch) L->disc.init_stochastic((uint32_t)c->seed, (size_t)(c->num_threads > 0 ? c->num_threads : 1));
  }
  return L;
}

void orc_learner_destroy(void* h) { delete (Learner*)h; }

// The by-node column sample of the following trees: fraction_bynode (>= 1: off), whether a by-tree
// sample is active (the by-node draw then picks among its features) and the sampler's LCG state
// after the host's by-tree draw.
void orc_learner_set_bynode(void* h, double fraction, int32_t bytree_active, uint32_t rng_state) {
  Learner* L = (Learner*)h;
  L->bynode_fraction = fraction;
  L->bytree_active = bytree_active != 0;
  L->node_rng.x = rng_state;
}

// The LCG state after the last tree's by-node draws.
uint32_t orc_learner_bynode_state(void* h) { return ((Learner*)h)->node_rng.x; }

// Interaction constraints: `num_sets` sets of real feature indices, set k at
// features[offsets[k] .. offsets[k + 1]); features the learner does not use are dropped.
void orc_learner_set_interaction_constraints(void* h, const int32_t* features, const int32_t* offsets,
                                             int32_t num_sets) {
  Learner* L = (Learner*)h;
  L->icons.clear();
  for (int32_t k = 0; k < num_sets; ++k) {
    std::vector<uint8_t> c((size_t)L->nf, 0);
    for (int32_t i = offsets[k]; i < offsets[k + 1]; ++i)
      for (int32_t f = 0; f < L->nf; ++f)
        if (L->metas[(size_t)f].real == features[i]) c[(size_t)f] = 1;
    L->icons.push_back(c);
  }
}

// The features the following trees may split on (ColSampler::reset_by_tree, col_sampler.rs:87-103):
// mask[f] != 0 for every used inner feature f; NULL restores "all features".
void orc_learner_set_feature_mask(void* h, const uint8_t* mask) {
  Learner* L = (Learner*)h;
  if (mask) L->tree_mask.assign(mask, mask + L->nf);
  else L->tree_mask.clear();
}

// Trains one tree. Returns the number of leaves; fills `splits` (num_leaves-1 capacity) and
// `leaf_value` (num_leaves capacity, the tree's leaf outputs before shrinkage).
int32_t orc_learner_train(void* h, const float* g, const float* hs, const int32_t* rows, int64_t nrows,
                          orc_split* splits, double* leaf_value) {
  Learner* L = (Learner*)h;
  L->train(g, hs, rows, nrows);
  for (size_t i = 0; i < L->records.size(); ++i) splits[i] = L->records[i];
  for (int32_t i = 0; i < L->tree_leaves; ++i) leaf_value[i] = L->leaf_value[i];
  return L->tree_leaves;
}

// Root output of the last tree (tree.rs set_leaf_output of leaf 0 before any split).
double orc_learner_root_output(void* h) { return ((Learner*)h)->root_output; }

// Leaf of every row after the last tree (-1 for rows outside the bagged set).
void orc_learner_row_leaf(void* h, int32_t* out) {
  Learner* L = (Learner*)h;
  for (int64_t i = 0; i < L->n; ++i) out[i] = -1;
  for (int32_t leaf = 0; leaf < L->tree_leaves; ++leaf) {
    const int32_t* ix = L->leaf_rows(leaf);
    for (int64_t k = 0; k < L->leaf_count[leaf]; ++k) out[ix[k]] = leaf;
  }
}

// The worker threads of the per-feature tasks and the block partition (the reference's rayon
// pool size). Independent of config num_threads, which also seeds the stochastic-rounding noise
// blocks (gradient_discretizer/mod.rs:87-106) and so stays what the reference run used.
void orc_learner_set_threads(void* h, int32_t threads) {
  Learner* L = (Learner*)h;
  delete L->workers;
  L->workers = new Pool(threads > 0 ? threads : 1);
}

// serial.rs:1974-1990 — SerialTreeLearner::add_prediction_to_score: every row of leaf l of the
// last tree gets score[row] += leaf_values[l] (leaf_values: the tree's values after shrinkage).
void orc_learner_add_score(void* h, const double* leaf_values, double* score) {
  Learner* L = (Learner*)h;
  if (L->tree_leaves <= 1) return;
  for (int32_t leaf = 0; leaf < L->tree_leaves; ++leaf) {
    const int32_t* ix = L->leaf_rows(leaf);
    const double out = leaf_values[leaf];
    for (int64_t k = 0; k < L->leaf_count[leaf]; ++k) score[ix[k]] += out;
  }
}

// The histogram pool slot of one leaf after the last tree ([total group bins][2] (gradient,
// hessian): double on the float path, int64 on the quantized path), or -1 when the leaf has no slot.
// used_out [nf]: 1 for the features of the leaf's last search, whose entries the slot holds.
int32_t orc_learner_leaf_histogram(void* h, int32_t leaf, void* out, uint8_t* used_out) {
  Learner* L = (Learner*)h;
  if (leaf < 0 || leaf >= L->num_leaves) return -1;
  const int32_t slot = L->leaf_slot[(size_t)leaf];
  if (slot < 0) return -1;
  std::copy(L->leaf_used[(size_t)leaf].begin(), L->leaf_used[(size_t)leaf].end(), used_out);
  for (int64_t b = 0; b < L->total_bins; ++b) {
    if (L->quant) {
      reinterpret_cast<int64_t*>(out)[2 * b] = L->islots_g[(size_t)slot][(size_t)b];
      reinterpret_cast<int64_t*>(out)[2 * b + 1] = L->islots_h[(size_t)slot][(size_t)b];
    } else {
      reinterpret_cast<double*>(out)[2 * b] = L->slots[(size_t)slot][(size_t)(2 * b)];
      reinterpret_cast<double*>(out)[2 * b + 1] = L->slots[(size_t)slot][(size_t)(2 * b + 1)];
    }
  }
  return slot;
}

// Partition order (indices) and per-leaf ranges after the last tree.
void orc_learner_partition(void* h, int32_t* indices, int64_t* begin, int64_t* count) {
  Learner* L = (Learner*)h;
  std::copy(L->indices.begin(), L->indices.end(), indices);
  for (int32_t i = 0; i < L->num_leaves; ++i) {
    begin[i] = L->leaf_begin[i];
    count[i] = L->leaf_count[i];
  }
}

// Packed quantized gradients of the last tree and the scales.
void orc_learner_packed(void* h, int16_t* out, double* scales) {
  Learner* L = (Learner*)h;
  if (!L->quant) return;
  std::copy(L->disc.packed.begin(), L->disc.packed.end(), out);
  scales[0] = L->gscale;
  scales[1] = L->hscale;
}

// Root-leaf histogram primitives (all rows), for kernel-level parity tests.
// Float: out[2*total_bins] per feature slices as the learner lays them out (group bins).
void orc_hist_float(const uint8_t* bins_colmajor, int64_t n, int32_t nf, const int32_t* group_bins,
                    const int32_t* rows, int64_t nrows, const float* g, const float* h, int32_t const_hess,
                    double* out) {
  int64_t cur = 0;
  for (int f = 0; f < nf; ++f) {
    double* o = out + 2 * cur;
    std::fill(o, o + 2 * group_bins[f], 0.0);
    const uint8_t* col = bins_colmajor + (size_t)f * (size_t)n;
    for (int64_t i = 0; i < nrows; ++i) {
      int64_t r = rows ? rows[i] : i;
      size_t ti = (size_t)col[r] << 1;
      o[ti] += (double)g[r];
      o[ti + 1] += const_hess ? 1.0 : (double)h[r];
    }
    if (const_hess && n > 0)  // hessians[0] exists only for a non-empty dataset
      for (int b = 0; b < group_bins[f]; ++b) o[2 * b + 1] *= (double)h[0];
    cur += group_bins[f];
  }
}

void orc_hist_int(const uint8_t* bins_colmajor, int64_t n, int32_t nf, const int32_t* group_bins,
                  const int32_t* rows, int64_t nrows, const int16_t* packed, int64_t* out_g, int64_t* out_h) {
  int64_t cur = 0;
  for (int f = 0; f < nf; ++f) {
    std::fill(out_g + cur, out_g + cur + group_bins[f], 0);
    std::fill(out_h + cur, out_h + cur + group_bins[f], 0);
    const uint8_t* col = bins_colmajor + (size_t)f * (size_t)n;
    for (int64_t i = 0; i < nrows; ++i) {
      int64_t r = rows ? rows[i] : i;
      int b = col[r];
      out_g[cur + b] += (int64_t)(int8_t)(packed[r] >> 8);
      out_h[cur + b] += (int64_t)(uint8_t)(packed[r] & 0xff);
    }
    cur += group_bins[f];
  }
}

// Discretization alone (gradient_discretizer/mod.rs), for the golden vectors.
int32_t orc_discretize(const float* g, const float* h, int64_t n, int32_t bins, int32_t const_hess,
                       int32_t stochastic, uint32_t seed, int32_t num_threads, int32_t fused, int32_t calls,
                       int16_t* out, double* scales) {
  Discretizer d;
  d.init((size_t)n, bins, const_hess != 0, fused != 0);
  if (stochastic) d.init_stochastic(seed, (size_t)(num_threads > 0 ? num_threads : 1));
  bool ok = true;
  for (int c = 0; c < calls; ++c) ok = stochastic ? d.discretize_stochastic(g, h) : d.discretize_nearest(g, h);
  std::copy(d.packed.begin(), d.packed.end(), out);
  scales[0] = d.gscale;
  scales[1] = d.hscale;
  return ok ? 1 : 0;
}

// mt19937 draws: kind 0 = raw u32, 1 = uniform_real_01 bits, 2 = uniform_int_inclusive(arg).
void orc_mt19937(uint32_t seed, int32_t kind, uint32_t arg, int64_t count, uint64_t* out) {
  Mt19937 e(seed);
  for (int64_t i = 0; i < count; ++i) {
    if (kind == 0) out[i] = e.next_u32();
    else if (kind == 1) {
      double v = e.uniform_real_01();
      uint64_t b;
      std::memcpy(&b, &v, 8);
      out[i] = b;
    } else out[i] = e.uniform_int_inclusive(arg);
  }
}

// Route table of one numerical split (data_partition.rs:299-410) for a single-feature group.
void orc_route_table(const orc_feature* f, uint32_t threshold, int32_t default_left, uint8_t* lut) {
  FeatureMeta m;
  m.num_bin = f->num_bin;
  m.missing = f->missing_type;
  m.default_bin = f->default_bin;
  m.mfb = f->most_freq_bin;
  m.offset = m.mfb == 0 ? 1 : 0;
  m.penalty = f->penalty;
  m.real = f->real_feature;
  route_table(m, threshold, default_left != 0, 1 + m.num_bin - m.offset, lut);
}

int32_t orc_sizeof_split(void) { return (int32_t)sizeof(orc_split); }

static Params params_of(const orc_config* c) {
  Params p;
  p.l1 = c->lambda_l1;
  p.l2 = c->lambda_l2;
  p.max_delta = c->max_delta_step;
  p.smooth = c->path_smooth;
  p.min_data = c->min_data_in_leaf;
  p.min_hess = c->min_sum_hessian_in_leaf;
  p.min_gain = c->min_gain_to_split;
  p.fused = c->fused_madd != 0;
  p.max_cat_to_onehot = c->max_cat_to_onehot;
  p.max_cat_threshold = c->max_cat_threshold;
  p.cat_smooth = c->cat_smooth;
  p.cat_l2 = c->cat_l2;
  p.min_data_per_group = c->min_data_per_group;
  return p;
}

static FeatureMeta meta_of(const orc_feature* f) {
  FeatureMeta m;
  m.num_bin = f->num_bin;
  m.missing = f->missing_type;
  m.default_bin = f->default_bin;
  m.mfb = f->most_freq_bin;
  m.offset = m.mfb == 0 ? 1 : 0;
  m.penalty = f->penalty;
  m.real = f->real_feature;
  m.categorical = f->bin_type == 1 ? 1 : 0;
  return m;
}

// One integer threshold search (feature_histogram.rs:673) on a feature-local histogram of
// num_bin - offset bins. Result written as a split record (threshold, counts, outputs, sums, gain,
// default_left, int sums); returns the splittable flag.
int32_t orc_find_best_threshold_int(const int64_t* hg, const int64_t* hh, const orc_feature* f,
                                    const orc_config* c, int64_t tg, int64_t th, double gs, double hs,
                                    int32_t num_data, double parent_output, orc_split* out) {
  FeatureMeta m = meta_of(f);
  Params p = params_of(c);
  SplitInfo si;
  bool sp = find_best_threshold_numerical_int(hg, hh, m, p, tg, th, gs, hs, num_data, parent_output, &si);
  std::memset(out, 0, sizeof(*out));
  out->threshold = si.threshold;
  out->default_left = si.default_left;
  out->left_count = si.left_count;
  out->right_count = si.right_count;
  out->left_output = si.left_output;
  out->right_output = si.right_output;
  out->left_sum_gradient = si.lsg;
  out->left_sum_hessian = si.lsh;
  out->right_sum_gradient = si.rsg;
  out->right_sum_hessian = si.rsh;
  out->gain = si.gain;
  out->left_int_sum = si.lint;
  out->right_int_sum = si.rint;
  return sp ? 1 : 0;
}

// One float threshold search (feature_histogram.rs:219) on a feature-local [g, h] histogram.
int32_t orc_find_best_threshold(const double* hist, const orc_feature* f, const orc_config* c, double sg,
                                double sh, int32_t num_data, double parent_output, orc_split* out) {
  FeatureMeta m = meta_of(f);
  Params p = params_of(c);
  SplitInfo si;
  bool sp = find_best_threshold_numerical(hist, m, p, sg, sh, num_data, parent_output, &si);
  std::memset(out, 0, sizeof(*out));
  out->threshold = si.threshold;
  out->default_left = si.default_left;
  out->left_count = si.left_count;
  out->right_count = si.right_count;
  out->left_output = si.left_output;
  out->right_output = si.right_output;
  out->left_sum_gradient = si.lsg;
  out->left_sum_hessian = si.lsh;
  out->right_sum_gradient = si.rsg;
  out->right_sum_hessian = si.rsh;
  out->gain = si.gain;
  return sp ? 1 : 0;
}

// Route table of one categorical split (bits: the bin bitset of the split, 8 words).
void orc_route_table_cat(const orc_feature* f, const uint32_t* bits, uint8_t* lut) {
  FeatureMeta m = meta_of(f);
  route_table_cat(m, bits, 1 + m.num_bin - m.offset, lut);
}

}  // extern "C"

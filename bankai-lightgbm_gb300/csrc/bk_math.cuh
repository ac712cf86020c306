// Split-gain and leaf-output arithmetic on the device, in the reference's operation order
// (treelearner/feature_histogram.rs:58-176, simd.rs:6-8). The translation units are compiled
// with -fmad=false, so no multiply-add is contracted; the reference's one deliberate fused
// multiply-add (`madd`, utils/common.rs:207-216) is `fma()` when Params::fused is set.
#pragma once
#include "bk_common.cuh"

namespace bk {

__device__ __forceinline__ double sgn(double x) { return (double)((int)(x > 0.0) - (int)(x < 0.0)); }

// feature_histogram.rs:66 — static_cast<int>(x + 0.5), saturating like Rust's `as i32`.
__device__ __forceinline__ int32_t round_int(double x) { return __double2int_rz(x + 0.5); }

__device__ __forceinline__ double threshold_l1(double s, double l1) {
  double reg = fmax(fabs(s) - l1, 0.0);
  return sgn(s) * reg;
}

__device__ __forceinline__ double madd(double a, double b, double c, bool fused) {
  if (fused) return fma(a, b, c);
  double q = a * b;
  return q + c;
}

// feature_histogram.rs:79-104 — CalculateSplittedLeafOutput<L1, MAX_OUT, SMOOTH>.
__device__ __forceinline__ double leaf_output(bool l1f, bool mxf, bool smf, double sg, double sh, const Params& p,
                                              int32_t n, double parent) {
  double ret;
  if (l1f) {
    double t = -threshold_l1(sg, p.l1);
    ret = t / (sh + p.l2);
  } else {
    double t = -sg;
    ret = t / (sh + p.l2);
  }
  if (mxf && p.max_delta > 0.0 && fabs(ret) > p.max_delta) ret = sgn(ret) * p.max_delta;
  if (smf) {
    double nn = (double)n;
    double a = nn / p.smooth;
    double t1 = ret * a;
    t1 = t1 / (a + 1.0);
    double t2 = parent / (a + 1.0);
    ret = t1 + t2;
  }
  return ret;
}

// feature_histogram.rs:127-144 — GetLeafGainGivenOutput.
__device__ __forceinline__ double leaf_gain_given_output(bool l1f, double sg, double sh, const Params& p, double out) {
  double g = l1f ? threshold_l1(sg, p.l1) : sg;
  double hl = sh + p.l2;
  double q = hl * out;
  q = q * out;
  return -madd(2.0 * g, out, q, p.fused != 0);
}

// feature_histogram.rs:148-176 — GetLeafGain.
__device__ __forceinline__ double leaf_gain(const Params& p, double sg, double sh, int32_t n, double parent) {
  const bool l1f = p.use_l1, mxf = p.use_max, smf = p.use_smooth;
  if (!mxf && !smf) {
    if (l1f) {
      double s = threshold_l1(sg, p.l1);
      double q = s * s;
      return q / (sh + p.l2);
    }
    double q = sg * sg;
    return q / (sh + p.l2);
  }
  double out = leaf_output(l1f, mxf, smf, sg, sh, p, n, parent);
  return leaf_gain_given_output(l1f, sg, sh, p, out);
}

// simd.rs:6-8 plus feature_histogram.rs:440-466.
__device__ __forceinline__ double split_gains(const Params& p, double slg, double slh, double srg, double srh,
                                              int32_t lc, int32_t rc, double parent) {
  if (!p.use_l1 && !p.use_max && !p.use_smooth) {
    double a = slg * slg;
    a = a / (slh + p.l2);
    double b = srg * srg;
    b = b / (srh + p.l2);
    return a + b;
  }
  double a = leaf_gain(p, slg, slh, lc, parent);
  double b = leaf_gain(p, srg, srh, rc, parent);
  return a + b;
}

__device__ __forceinline__ double split_output(const Params& p, double sg, double sh, int32_t n, double parent) {
  return leaf_output(p.use_l1, p.use_max, p.use_smooth, sg, sh, p, n, parent);
}

// feature_histogram.rs:114-125 — the root / parent output, <L1=true, MAX=true, SMOOTH=false>.
__device__ __forceinline__ double leaf_output_root(const Params& p, double sg, double sh, int32_t n) {
  double r = leaf_output(true, true, false, sg, sh, p, n, 0.0);
  if (isnan(r)) return r;
  return fmin(fmax(r, -1.7976931348623157e308), 1.7976931348623157e308);
}

__device__ __forceinline__ double round_to_zero(double v) {  // tree.rs:66-68
  return (v >= -BK_ZERO_THRESHOLD && v <= BK_ZERO_THRESHOLD) ? 0.0 : v;
}

// split_info.rs:104-121 — higher gain, then the smaller real feature (-1 counts as largest).
__device__ __forceinline__ bool better_than(double ga, int32_t fa, double gb, int32_t fb) {
  if (ga != gb) return ga > gb;
  int32_t a = fa == -1 ? 0x7fffffff : fa;
  int32_t b = fb == -1 ? 0x7fffffff : fb;
  return a < b;
}

// The route of one stored bin for a numerical split of a single-feature dense group
// (data_partition.rs:299-410 with group_view :25-40: min_bin 1, max_bin gbins - 1,
// use_min_bin false). 1 = left.
__device__ __forceinline__ uint8_t route_bin(const DevFeature& m, uint32_t threshold, bool default_left, uint32_t bin) {
  const uint32_t min_bin = 1, max_bin = (uint32_t)m.gbins - 1;
  const uint32_t default_bin = (uint32_t)m.default_bin, mfb = (uint32_t)m.mfb;
  bool miss_zero = false, miss_na = false, mfb_zero = false, mfb_na = false;
  if (m.missing == 1) {
    miss_zero = true;
    mfb_zero = default_bin == mfb;
  } else if (m.missing == 2) {
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
  const bool either_mfb = (miss_na && mfb_na) || (miss_zero && mfb_zero);
  bool left;
  if (min_bin < max_bin) {
    if ((miss_zero && !mfb_zero && bin == t_zero_bin) || (miss_na && !mfb_na && bin == max_bin))
      left = missing_default_left;
    else if (bin == 0)
      left = either_mfb ? missing_default_left : default_route_left;
    else
      left = !(bin > th);
  } else if (miss_zero && !mfb_zero && bin == t_zero_bin) {
    left = missing_default_left;
  } else if (bin != max_bin) {
    left = either_mfb ? missing_default_left : default_route_left;
  } else if (miss_na && !mfb_na) {
    left = missing_default_left;
  } else {
    left = max_bin_left;
  }
  return left ? 1 : 0;
}

}  // namespace bk

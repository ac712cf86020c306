// FindBestSplitsFromHistograms (serial.rs:1322-1566, int: :1212-1300) and the grow-loop
// bookkeeping kernels (serial.rs:578-628, :779-825, :1685-1876), GB300 form.
//
// k_search: one warp per (leaf, feature). It fixes the smaller leaf's most-frequent bin
// (FixHistogram, serial.rs:2205-2238), derives the larger leaf by parent-minus-smaller
// subtraction in place, then runs the reference's directional threshold scans
// (FindBestThresholdSequentially[Int], feature_histogram.rs:363-663 / 839-1142) as warp-parallel
// prefix scans over 32 thresholds at a time. The sequential scan's `break` (the first threshold
// whose other side falls under min_data / min_hessian ends the scan) becomes "the first such
// position in scan order and everything after it is excluded"; `current_gain > best_gain` becomes
// a warp argmax with ties going to the earliest position in scan order. The quantized path's
// prefix sums are exact integers, so its candidates are bit-identical to the reference's; the
// float path's f64 prefix sums are associated differently (≈1e-16 relative).
//
// The last CTA of k_search folds the per-feature candidates of each searched leaf in feature
// order with `better_than`, takes the arg-max leaf (split_info.rs:88-96), stops the tree when its
// gain is <= 0, and builds the route table of the chosen split (data_partition.rs:299-410). The
// post-split bookkeeping (bk_grow.cuh) runs in the last CTA of the partition scatter.
#include <math_constants.h>

#include "bk_grow.cuh"
#include "bk_math.cuh"

namespace bk {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

struct DirBest {
  int splittable;
  double gain;      // best gain of this direction (-inf when none)
  int32_t th, lc;
  double slg, slh;  // float path
  int64_t lg, lh;   // int path
};

// Accessors of one feature's slice in a pool slot: local bin t lives at group bin t + 1.
struct FloatHist {
  double2* base;  // entry of group bin 0 of this feature
  __device__ double2 get(int t) const { return base[(size_t)(t + 1) * TILE]; }
};
struct IntHist {
  int64_t* base;
  __device__ int64_t get(int t) const { return base[(size_t)(t + 1) * TILE]; }
};

__device__ __forceinline__ int64_t unpack_g(int64_t pk) { return pk >> 32; }
__device__ __forceinline__ int64_t unpack_h(int64_t pk) { return pk & 0xffffffffLL; }

// Warp arg-max over lanes whose candidate beats `cur`; ties go to the lowest lane.
__device__ __forceinline__ int warp_best_lane(bool better, double gain, int lane, double* out_gain) {
  double bg = better ? gain : -CUDART_INF;
  int bl = better ? lane : 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double og = __shfl_xor_sync(FULL, bg, o);
    int ol = __shfl_xor_sync(FULL, bl, o);
    if (og > bg || (og == bg && ol < bl)) {
      bg = og;
      bl = ol;
    }
  }
  *out_gain = bg;
  return bl;
}

// ---- fp32 prefilter of the plain split gain (no L1 / max_delta_step / path_smooth) ----
// The reference evaluates gl^2/(hl+l2) + gr^2/(hr+l2) in f64 for every threshold; GB300 runs f64 at
// a small fraction of its fp32 rate. Each candidate is first evaluated in fp32 together with a
// rigorous bound E on |fp32 - f64| (the inputs' conversion, the squares, the sums and the division
// add up to about 14 units of 2^-24 relative to the non-negative result, the fp32 comparisons
// against E one more; E uses 48). Only the
// candidates that can still be the best (fp32 + E >= the best lower bound so far) or whose
// pass/fail against min_gain_shift is uncertain are evaluated in f64, so the chosen split, its
// gain and the splittable flag are exactly the reference's.
constexpr float kPrefilterRel = 48.0f * 5.9604645e-08f;

struct Approx {
  float g, e;
  bool uncertain;
};

__device__ __forceinline__ Approx approx_from(float xl, float yl, float xr, float yr) {
  Approx a;
  float tl = __fdiv_rn(__fmul_rn(xl, xl), yl);
  float tr = __fdiv_rn(__fmul_rn(xr, xr), yr);
  a.g = __fadd_rn(tl, tr);
  a.e = __fadd_rn(__fmul_rn(kPrefilterRel, a.g), 1e-30f);
  // non-finite values, tiny denominators (where the reference's +kEpsilon matters) and huge
  // numerators go to f64
  a.uncertain = !(yl >= 1e-6f) || !(yr >= 1e-6f) || !(a.g < 1e30f) || isnan(a.g);
  return a;
}

// Smallest x in [0, hi) with pred(x) (monotone false -> true), or hi; one warp, 32-ary search.
template <typename Pred>
__device__ int64_t warp_first_true(int64_t hi, int lane, Pred pred) {
  int64_t lo = 0;
  while (lo < hi) {
    int64_t step = (hi - lo + 31) / 32;
    int64_t x = lo + (int64_t)lane * step;
    bool t = x < hi && pred(x);
    unsigned m = __ballot_sync(FULL, t);
    if (m == 0) {
      int64_t nlo = lo + 31 * step + 1;
      lo = nlo < hi ? nlo : hi;
    } else {
      int k = __ffs(m) - 1;
      hi = lo + (int64_t)k * step;
      if (k > 0) lo = lo + (int64_t)(k - 1) * step + 1;
    }
  }
  return lo;
}

// FindBestThresholdSequentially (float), feature_histogram.rs:363-663.
template <bool REV, bool PLAIN>
__device__ DirBest scan_float(const Params& p, const DevFeature& m, const FloatHist& H, bool SKIP, bool NA,
                              double sum_g, double sum_h, int32_t num_data, double mgs, double parent, int lane) {
  DirBest r;
  r.splittable = 0;
  r.gain = -CUDART_INF;
  r.th = m.num_bin;
  r.lc = 0;
  r.slg = CUDART_NAN;
  r.slh = CUDART_NAN;
  r.lg = r.lh = 0;
  const double cnt_factor = (double)num_data / sum_h;
  const int off = m.offset;
  const float l2f = (float)p.l2;
  const float mgs_up = __double2float_ru(mgs), mgs_dn = __double2float_rd(mgs);
  double cg, ch;
  int32_t cc;
  int t_first, P;
  if (REV) {
    t_first = m.num_bin - 1 - off - (NA ? 1 : 0);
    int t_end = 1 - off;
    P = t_first - t_end + 1;
    cg = 0.0;
    ch = BK_EPS;
    cc = 0;
  } else {
    int t_end = m.num_bin - 2 - off;
    if (NA && off == 1) {
      // left starts as everything outside the slice (the most-frequent bin 0)
      double pg = 0.0, ph = 0.0;
      int32_t pc = 0;
      for (int i = lane; i < m.num_bin - off; i += 32) {
        double2 v = H.get(i);
        pg += v.x;
        ph += v.y;
        pc += round_int(v.y * cnt_factor);
      }
      pg = warp_sum(pg);
      ph = warp_sum(ph);
      pc = warp_sum(pc);
      cg = sum_g - pg;
      ch = (sum_h - BK_EPS) - ph;
      cc = num_data - pc;
      t_first = -1;
    } else {
      cg = 0.0;
      ch = BK_EPS;
      cc = 0;
      t_first = 0;
    }
    P = t_end - t_first + 1;
  }
  for (int c0 = 0; c0 < P; c0 += 32) {
    int k = c0 + lane;
    int t = REV ? t_first - k : t_first + k;
    bool act = k < P;
    bool cand = act && !(SKIP && (t + off) == m.default_bin);
    double g = 0.0, h = 0.0;
    int32_t c = 0;
    if (cand && t >= 0) {
      double2 v = H.get(t);
      g = v.x;
      h = v.y;
      c = round_int(h * cnt_factor);
    }
    double pg = warp_incl_scan(g, lane) + cg;
    double ph = warp_incl_scan(h, lane) + ch;
    int32_t pc = warp_incl_scan(c, lane) + cc;
    cg = __shfl_sync(FULL, pg, 31);
    ch = __shfl_sync(FULL, ph, 31);
    cc = __shfl_sync(FULL, pc, 31);
    bool first, brk;
    double slg, slh, srg, srh;
    int32_t lc, rc;
    if (REV) {
      srg = pg;
      srh = ph;
      rc = pc;
      first = cand && !(rc < p.min_data || srh < p.min_hess);
      lc = num_data - rc;
      slh = sum_h - srh;
      brk = first && (lc < p.min_data || slh < p.min_hess);
      slg = sum_g - srg;
    } else {
      slg = pg;
      slh = ph;
      lc = pc;
      first = cand && !(lc < p.min_data || slh < p.min_hess);
      rc = num_data - lc;
      srh = sum_h - slh;
      brk = first && (rc < p.min_data || srh < p.min_hess);
      srg = sum_g - slg;
    }
    unsigned bm = __ballot_sync(FULL, brk);
    int stop_lane = bm ? __ffs(bm) - 1 : 32;
    bool valid = first && !brk && lane < stop_lane;
    bool exact = valid, cpass = false;
    if (PLAIN) {
      Approx a{0.f, 0.f, true};
      if (valid) a = approx_from((float)slg, __fadd_rn((float)slh, l2f), (float)srg, __fadd_rn((float)srh, l2f));
      float e2 = a.e;
      cpass = valid && !a.uncertain && __fsub_rn(a.g, e2) > mgs_up;
      bool mpass = valid && (a.uncertain || __fadd_rn(a.g, e2) > mgs_dn);
      float lower = cpass ? __fsub_rn(a.g, e2) : -CUDART_INF_F;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lower = fmaxf(lower, __shfl_xor_sync(FULL, lower, o));
      float thr = fmaxf(lower, __double2float_rd(r.gain));
      bool contender = mpass && (a.uncertain || __fadd_rn(a.g, e2) >= thr);
      bool any_cpass = __any_sync(FULL, cpass);
      bool unsure = mpass && !cpass && !any_cpass && !r.splittable;
      exact = contender || unsure;
    }
    double gain = exact ? split_gains(p, slg, slh, srg, srh, lc, rc, parent) : -CUDART_INF;
    bool pass = exact ? !(gain <= mgs) : cpass;
    if (__any_sync(FULL, valid && pass)) r.splittable = 1;
    double bg;
    int bl = warp_best_lane(exact && pass && gain > r.gain, gain, lane, &bg);
    if (bl < 32) {
      r.gain = bg;
      r.th = __shfl_sync(FULL, REV ? (t - 1 + off) : (t + off), bl);
      r.lc = __shfl_sync(FULL, lc, bl);
      r.slg = __shfl_sync(FULL, slg, bl);
      r.slh = __shfl_sync(FULL, slh, bl);
    }
    if (bm) break;
  }
  return r;
}

// As warp_first_true, trying first the 32 values around `guess` (one warp-wide evaluation) and
// falling back to the full search when the answer lies outside that window.
template <typename Pred>
__device__ int64_t warp_first_true_near(int64_t hi, int64_t guess, int lane, Pred pred) {
  guess = guess < 0 ? 0 : (guess > hi ? hi : guess);
  const int64_t x = guess - 15 + lane;
  const bool t = x >= hi ? true : (x < 0 ? false : pred(x));
  const unsigned m = __ballot_sync(FULL, t);
  if (m != 0u && (m & 1u) == 0u) return guess - 15 + (__ffs(m) - 1);  // false -> true inside
  if (m != 0u && guess - 15 <= 0) return 0;  // everything from 0 on is true
  return warp_first_true(hi, lane, pred);
}

// Integer thresholds of a leaf (feature-independent): for an accumulated side with integer hessian
// x, the reference's `count >= min_data && hess >= min_hessian` test (counts estimated as
// round_int(x * cnt_factor), feature_histogram.rs:927-940) is monotone in x, so it is x >= first_x;
// and the `break` test on the other side is x >= brk_x.
struct IntThresholds {
  int64_t first_x, brk_x;
};

__device__ IntThresholds int_thresholds(const Params& p, int64_t th, double hs, int32_t num_data, int lane) {
  const double cf = (double)num_data / (double)th;
  const int64_t hi = th + 1;
  // fp32 guesses of the transitions; the exact f64 predicates decide
  const float fth = (float)th, fnd = (float)num_data;
  const int64_t g_cnt = (int64_t)((float)((double)p.min_data - 0.5) * fth / fnd);
  const int64_t g_brk = (int64_t)((float)((double)(num_data - p.min_data) + 0.5) * fth / fnd);
  const float fh = (float)hs;
  const int64_t g_hess = fh > 0.f ? (int64_t)fminf((float)p.min_hess / fh, 4.0e18f) : hi;
  int64_t cnt_ok = warp_first_true_near(hi, g_cnt, lane,
                                        [&](int64_t x) { return round_int((double)x * cf) >= p.min_data; });
  int64_t hess_ok = warp_first_true_near(hi, g_hess, lane, [&](int64_t x) { return (double)x * hs >= p.min_hess; });
  int64_t cnt_brk = warp_first_true_near(
      hi, g_brk, lane, [&](int64_t x) { return round_int((double)x * cf) > num_data - p.min_data; });
  IntThresholds r;
  r.first_x = cnt_ok > hess_ok ? cnt_ok : hess_ok;
  int64_t hess_brk = th - hess_ok + 1;  // (th - x) * hs < min_hess  <=>  th - x < hess_ok
  r.brk_x = cnt_brk < hess_brk ? cnt_brk : hess_brk;
  return r;
}

// FindBestThresholdSequentiallyInt, feature_histogram.rs:839-1142. With PLAIN gains the scan
// runs twice over the (cheap, exact) integer prefix sums: pass 1 evaluates every threshold in
// fp32 and finds the best certified lower bound M; pass 2 evaluates in f64 only the thresholds
// whose upper bound reaches M (plus, while the splittable flag is still undecided, those whose
// pass / fail is uncertain), so most 32-threshold chunks take no f64 instruction at all.
template <bool REV, bool PLAIN>
__device__ DirBest scan_int(const Params& p, const DevFeature& m, const IntHist& H, bool SKIP, bool NA, int64_t tg,
                            int64_t th, double gs, double hs, int32_t num_data, double mgs, double parent,
                            const IntThresholds& X, int lane) {
  DirBest r;
  r.splittable = 0;
  r.gain = -CUDART_INF;
  r.th = m.num_bin;
  r.lc = 0;
  r.slg = r.slh = 0.0;
  r.lg = r.lh = 0;
  const double cnt_factor = (double)num_data / (double)th;
  const int off = m.offset;
  const float gsf = (float)gs, hsf = (float)hs, l2f = (float)p.l2;
  const float mgs_up = __double2float_ru(mgs), mgs_dn = __double2float_rd(mgs);
  int64_t cg0, ch0;
  int t_first, P;
  if (REV) {
    t_first = m.num_bin - 1 - off - (NA ? 1 : 0);
    P = t_first - (1 - off) + 1;
    cg0 = ch0 = 0;
  } else {
    int t_end = m.num_bin - 2 - off;
    if (NA && off == 1) {
      int64_t pg = 0, ph = 0;
      for (int i = lane; i < m.num_bin - off; i += 32) {
        int64_t v = H.get(i);
        pg += unpack_g(v);
        ph += unpack_h(v);
      }
      cg0 = tg - warp_sum(pg);
      ch0 = th - warp_sum(ph);
      t_first = -1;
    } else {
      cg0 = ch0 = 0;
      t_first = 0;
    }
    P = t_end - t_first + 1;
  }
  // pass 1 (PLAIN only): the best certified lower bound, and whether some threshold certainly passes
  float M = -CUDART_INF_F;
  bool certain_split = false;
  const int passes = PLAIN ? 2 : 1;
  for (int pass = 0; pass < passes; ++pass) {
    const bool exact_pass = pass == passes - 1;
    int64_t cg = cg0, ch = ch0;
    for (int c0 = 0; c0 < P; c0 += 32) {
      int k = c0 + lane;
      int t = REV ? t_first - k : t_first + k;
      bool act = k < P;
      bool cand = act && !(SKIP && (t + off) == m.default_bin);
      int64_t g = 0, h = 0;
      if (cand && t >= 0) {
        int64_t v = H.get(t);
        g = unpack_g(v);
        h = unpack_h(v);
      }
      int64_t pg = warp_incl_scan(g, lane) + cg;
      int64_t ph = warp_incl_scan(h, lane) + ch;
      cg = __shfl_sync(FULL, pg, 31);
      ch = __shfl_sync(FULL, ph, 31);
      // REV accumulates the right side, FWD the left side
      int64_t lg = REV ? tg - pg : pg;
      int64_t lh = REV ? th - ph : ph;
      int64_t rg = tg - lg, rh = th - lh;
      bool first = cand && ph >= X.first_x;
      bool brk = first && ph >= X.brk_x;
      unsigned bm = __ballot_sync(FULL, brk);
      int stop_lane = bm ? __ffs(bm) - 1 : 32;
      bool valid = first && !brk && lane < stop_lane;
      bool exact = valid;
      bool cpass = false;
      if (PLAIN) {
        Approx a{0.f, 0.f, true};
        if (valid)
          a = approx_from(__fmul_rn((float)lg, gsf), __fadd_rn(__fmul_rn((float)lh, hsf), l2f),
                          __fmul_rn((float)rg, gsf), __fadd_rn(__fmul_rn((float)rh, hsf), l2f));
        cpass = valid && !a.uncertain && __fsub_rn(a.g, a.e) > mgs_up;
        bool mpass = valid && (a.uncertain || __fadd_rn(a.g, a.e) > mgs_dn);
        if (!exact_pass) {
          float lower = cpass ? __fsub_rn(a.g, a.e) : -CUDART_INF_F;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) lower = fmaxf(lower, __shfl_xor_sync(FULL, lower, o));
          M = fmaxf(M, lower);
          if (__any_sync(FULL, cpass)) certain_split = true;
          if (bm) break;
          continue;
        }
        bool contender = mpass && (a.uncertain || __fadd_rn(a.g, a.e) >= M);
        bool unsure = mpass && !cpass && !certain_split && !r.splittable;
        exact = contender || unsure;
        if (certain_split) r.splittable = 1;
      }
      double gain = -CUDART_INF;
      if (__any_sync(FULL, exact)) {
        if (exact) {
          double slh = (double)lh * hs, srh = (double)rh * hs;
          int32_t lc = PLAIN ? 0 : round_int((double)lh * cnt_factor);
          int32_t rc = PLAIN ? 0 : round_int((double)rh * cnt_factor);
          gain = split_gains(p, (double)lg * gs, slh + BK_EPS, (double)rg * gs, srh + BK_EPS, lc, rc, parent);
        }
      }
      bool passed = exact ? !(gain <= mgs) : cpass;
      if (__any_sync(FULL, valid && passed)) r.splittable = 1;
      double bg;
      int bl = warp_best_lane(exact && passed && gain > r.gain, gain, lane, &bg);
      if (bl < 32) {
        r.gain = bg;
        r.th = __shfl_sync(FULL, REV ? (t - 1 + off) : (t + off), bl);
        r.lg = __shfl_sync(FULL, lg, bl);
        r.lh = __shfl_sync(FULL, lh, bl);
      }
      if (bm) break;
    }
  }
  return r;
}

__device__ void cand_reset(Cand* c, int32_t real, int32_t inner) {
  c->gain = -CUDART_INF;
  c->left_output = c->right_output = 0.0;
  c->lsg = c->lsh = c->rsg = c->rsh = 0.0;
  c->lint = c->rint = 0;
  c->feature = real;
  c->inner = inner;
  c->threshold = 0;
  c->left_count = c->right_count = 0;
  c->default_left = 1;
  c->splittable = 0;
}

// FindBestThreshold (float) for one leaf: feature_histogram.rs:219-357.
template <bool PLAIN>
__device__ void search_leaf_float(const Params& p, const DevFeature& m, const FloatHist& H, const LeafSum& ls,
                                  double parent, int lane, Cand* out, double* out_gain, uint8_t* out_split,
                                  int32_t f) {
  const double sum_g = ls.sg;
  const double sum_h = ls.sh + 2.0 * BK_EPS;
  const int32_t num_data = ls.num_data;
  double gain_shift = leaf_gain(p, sum_g, sum_h, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  DirBest d[2];
  int nd;
  if (m.num_bin > 2 && m.missing != 0) {
    bool skip = m.missing == 1, na = m.missing == 2;
    d[0] = scan_float<true, PLAIN>(p, m, H, skip, na, sum_g, sum_h, num_data, mgs, parent, lane);
    d[1] = scan_float<false, PLAIN>(p, m, H, skip, na, sum_g, sum_h, num_data, mgs, parent, lane);
    nd = 2;
  } else {
    d[0] = scan_float<true, PLAIN>(p, m, H, false, false, sum_g, sum_h, num_data, mgs, parent, lane);
    nd = 1;
  }
  if (lane != 0) return;
  Cand c;
  cand_reset(&c, m.real, f);
  int sp = 0;
  for (int i = 0; i < nd; ++i) {
    const DirBest& r = d[i];
    sp |= r.splittable;
    if (r.splittable && r.gain > c.gain + mgs) {
      c.threshold = (uint32_t)r.th;
      c.left_output = split_output(p, r.slg, r.slh, r.lc, parent);
      c.left_count = r.lc;
      c.lsg = r.slg;
      c.lsh = r.slh - BK_EPS;
      c.right_output = split_output(p, sum_g - r.slg, sum_h - r.slh, num_data - r.lc, parent);
      c.right_count = num_data - r.lc;
      c.rsg = sum_g - r.slg;
      c.rsh = (sum_h - r.slh) - BK_EPS;
      c.gain = r.gain - mgs;
      c.default_left = i == 0 ? 1 : 0;
    }
  }
  if (nd == 1 && m.missing == 2) c.default_left = 0;
  c.gain *= m.penalty;
  c.splittable = sp;
  *out = c;
  *out_gain = c.gain;
  *out_split = (uint8_t)sp;
}

// FindBestThresholdInt for one leaf: feature_histogram.rs:673-830.
template <bool PLAIN>
__device__ void search_leaf_int(const Params& p, const DevFeature& m, const IntHist& H, const LeafSum& ls,
                                double gs, double hs, double parent, int lane, Cand* out, double* out_gain,
                                uint8_t* out_split, int32_t f) {
  const int64_t tg = ls.int_sum >> 32;
  const int64_t th = ls.int_sum & 0xffffffffLL;
  const int32_t num_data = ls.num_data;
  const double sum_g = (double)tg * gs;
  const double sum_h = (double)th * hs;
  double gain_shift = leaf_gain(p, sum_g, sum_h, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  const IntThresholds X = int_thresholds(p, th, hs, num_data, lane);
  DirBest d[2];
  int nd;
  if (m.num_bin > 2 && m.missing != 0) {
    bool skip = m.missing == 1, na = m.missing == 2;
    d[0] = scan_int<true, PLAIN>(p, m, H, skip, na, tg, th, gs, hs, num_data, mgs, parent, X, lane);
    d[1] = scan_int<false, PLAIN>(p, m, H, skip, na, tg, th, gs, hs, num_data, mgs, parent, X, lane);
    nd = 2;
  } else {
    d[0] = scan_int<true, PLAIN>(p, m, H, false, false, tg, th, gs, hs, num_data, mgs, parent, X, lane);
    nd = 1;
  }
  if (lane != 0) return;
  Cand c;
  cand_reset(&c, m.real, f);
  const double cnt_factor = (double)num_data / (double)th;
  int sp = 0;
  for (int i = 0; i < nd; ++i) {
    const DirBest& r = d[i];
    sp |= r.splittable;
    if (r.splittable && r.gain > c.gain + mgs) {
      int64_t rg = tg - r.lg, rh = th - r.lh;
      double slg = (double)r.lg * gs, slh = (double)r.lh * hs;
      double srg = (double)rg * gs, srh = (double)rh * hs;
      int32_t lc = round_int((double)r.lh * cnt_factor);
      int32_t rc = round_int((double)rh * cnt_factor);
      c.threshold = (uint32_t)r.th;
      c.left_output = split_output(p, slg, slh, lc, parent);
      c.left_count = lc;
      c.lsg = slg;
      c.lsh = slh;
      c.right_output = split_output(p, srg, srh, rc, parent);
      c.right_count = rc;
      c.rsg = srg;
      c.rsh = srh;
      c.lint = (int64_t)(((uint64_t)r.lg << 32) | ((uint64_t)r.lh & 0xffffffffull));
      c.rint = (int64_t)(((uint64_t)rg << 32) | ((uint64_t)rh & 0xffffffffull));
      c.gain = r.gain - mgs;
      c.default_left = i == 0 ? 1 : 0;
    }
  }
  if (nd == 1 && m.missing == 2) c.default_left = 0;
  c.gain *= m.penalty;
  c.splittable = sp;
  *out = c;
  *out_gain = c.gain;
  *out_split = (uint8_t)sp;
}

__device__ __forceinline__ double parent_output_of(const Params& p, const JobState* st, const LeafSum& ls) {
  // serial.rs:1924-1935 (GetParentOutput)
  if (st->tree_leaves == 1) return leaf_output_root(p, ls.sg, ls.sh, ls.num_data);
  return ls.weight;
}

__device__ void decide_body(const Job& J, const Params& p, const DevFeature* feats);

// One warp per (leaf side, feature): side 0 = the smaller leaf, side 1 = the larger leaf.
// Side 0 fixes the smaller leaf's most-frequent bin (FixHistogram, serial.rs:2205-2238); side 1
// derives the larger leaf as parent minus the fixed smaller histogram (serial.rs:1407-1437,
// :1218-1242) — it recomputes the fixed most-frequent bin itself with the same reduction, so the
// two warps never wait for each other. The last CTA to finish runs the fold / arg-max (k_decide).
template <bool PLAIN, bool QUANT>
__global__ void __launch_bounds__(64) k_search(const Job* __restrict__ jobs, Params p,
                                               const DevFeature* __restrict__ feats) {
  const Job& J = jobs[blockIdx.z];
  JobState* st = J.st;
  if (st->stop) return;  // uniform over the grid
  const int lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int side = w >= p.F ? 1 : 0;
  const int f = w - side * p.F;
  const int32_t leaf = side ? st->larger_leaf : st->smaller_leaf;
  if (st->do_search && f < p.F && J.used[f] && leaf >= 0) {
    const DevFeature m = feats[f];
    const size_t slot_stride = (size_t)p.T * p.B * TILE;
    const size_t feat_off = (size_t)(f / TILE) * p.B * TILE + (f % TILE);
    const LeafSum S = J.leaf_sum[st->smaller_leaf];
    const LeafSum ls = side ? J.leaf_sum[leaf] : S;
    const double parent = parent_output_of(p, st, ls);
    if (QUANT) {
      int64_t* pool = reinterpret_cast<int64_t*>(J.pool);
      IntHist HS{pool + (size_t)st->smaller_slot * slot_stride + feat_off};
      int64_t fixed = 0;
      if (m.mfb > 0) {
        int64_t acc = 0;
        for (int i = lane; i < m.num_bin; i += 32)
          if (i != m.mfb) acc += HS.get(i);
        acc = warp_sum(acc);
        // the packed leaf total (grad << 32) | hess equals grad * 2^32 + hess, so packed
        // arithmetic is exact componentwise
        fixed = S.int_sum - acc;
      }
      if (side == 0) {
        if (m.mfb > 0 && lane == 0) HS.base[(size_t)(m.mfb + 1) * TILE] = fixed;
        __syncwarp();
        search_leaf_int<PLAIN>(p, m, HS, ls, st->gscale, st->hscale, parent, lane, &J.cand[f], &J.cgain[f],
                               &J.csplit[f], f);
      } else {
        IntHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
        for (int i = lane; i < m.len; i += 32) {
          int64_t sv = (m.mfb > 0 && i == m.mfb) ? fixed : HS.get(i);
          HL.base[(size_t)(i + 1) * TILE] -= sv;
        }
        __syncwarp();
        search_leaf_int<PLAIN>(p, m, HL, ls, st->gscale, st->hscale, parent, lane, &J.cand[p.F + f],
                               &J.cgain[p.F + f], &J.csplit[p.F + f], f);
      }
    } else {
      double2* pool = reinterpret_cast<double2*>(J.pool);
      FloatHist HS{pool + (size_t)st->smaller_slot * slot_stride + feat_off};
      double2 fixed = make_double2(0.0, 0.0);
      if (m.mfb > 0) {
        double ag = 0.0, ah = 0.0;
        for (int i = lane; i < m.num_bin; i += 32)
          if (i != m.mfb) {
            double2 v = HS.get(i);
            ag += v.x;
            ah += v.y;
          }
        ag = warp_sum(ag);
        ah = warp_sum(ah);
        fixed = make_double2(S.sg - ag, S.sh - ah);
      }
      if (side == 0) {
        if (m.mfb > 0 && lane == 0) HS.base[(size_t)(m.mfb + 1) * TILE] = fixed;
        __syncwarp();
        search_leaf_float<PLAIN>(p, m, HS, ls, parent, lane, &J.cand[f], &J.cgain[f], &J.csplit[f], f);
      } else {
        FloatHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
        for (int i = lane; i < m.len; i += 32) {
          double2 a = HL.get(i);
          double2 b = (m.mfb > 0 && i == m.mfb) ? fixed : HS.get(i);
          HL.base[(size_t)(i + 1) * TILE] = make_double2(a.x - b.x, a.y - b.y);
        }
        __syncwarp();
        search_leaf_float<PLAIN>(p, m, HL, ls, parent, lane, &J.cand[p.F + f], &J.cgain[p.F + f],
                                 &J.csplit[p.F + f], f);
      }
    }
  }
  // the last CTA of this launch runs the fold and the leaf arg-max
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned t = atomicAdd(&st->search_done, 1u);
    last = t == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  decide_body(J, p, feats);
  if (threadIdx.x == 0) st->search_done = 0u;
}

// ---------------------------------------------------------------------------------------------
// k_decide
// ---------------------------------------------------------------------------------------------

// Combine two (index, gain, real feature) candidates of a fold or an arg-max. `a` is the one
// that comes first in the sequential order; `b` replaces it only when strictly better
// (split_info.rs:104-121); NaN gains never win (the sequential fold never adopts them).
__device__ __forceinline__ void pick(int& ai, double& ag, int& af, int bi, double bg, int bf) {
  if (bi < 0 || isnan(bg)) return;
  if (ai < 0 || better_than(bg, bf, ag, af) || (!better_than(ag, af, bg, bf) && bi < ai)) {
    ai = bi;
    ag = bg;
    af = bf;
  }
}

// Cand is 8-byte aligned and its size a multiple of 8 (not of 16): copy it in 8-byte words.
static_assert(sizeof(Cand) % 8 == 0 && alignof(Cand) == 8, "Cand is copied in 8-byte words");
__device__ __forceinline__ Cand load_cand_cg(const Cand* c) {
  Cand r;
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(c);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(Cand) / 8); ++i) dst[i] = __ldcg(src + i);
  return r;
}

// The fold of the searched leaves' candidates and the leaf arg-max (64 threads). Everything
// written by other CTAs of the search launch is read through L2 (__ldcg).
__device__ void decide_body(const Job& J, const Params& p, const DevFeature* feats) {
  JobState* st = J.st;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (st->do_search) {
    // serial.rs:1523-1558 — fold the candidates of each searched leaf in feature order.
    const int32_t leaf = warp == 0 ? st->smaller_leaf : st->larger_leaf;
    const int32_t slot = warp == 0 ? st->smaller_slot : st->larger_slot;
    if (leaf >= 0) {
      int bi = -1, bf = 0x7fffffff;
      double bg = -CUDART_INF;
      for (int f = lane; f < p.F; f += 32) {
        if (!J.used[f]) continue;
        J.splittable[(size_t)slot * p.F + f] = __ldcg(&J.csplit[warp * p.F + f]);
        pick(bi, bg, bf, f, __ldcg(&J.cgain[warp * p.F + f]), feats[f].real);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        int oi = __shfl_xor_sync(FULL, bi, o);
        double og = __shfl_xor_sync(FULL, bg, o);
        int of = __shfl_xor_sync(FULL, bf, o);
        pick(bi, bg, bf, oi, og, of);
      }
      if (lane == 0) {
        // the fold starts from SplitInfo::default (gain -inf, feature -1) and replaces it only
        // with a better candidate
        Cand best;
        cand_reset(&best, -1, -1);
        if (bi >= 0 && better_than(bg, bf, best.gain, best.feature)) best = load_cand_cg(&J.cand[warp * p.F + bi]);
        J.best[leaf] = best;
        J.bgain[leaf] = best.gain;
        J.bfeat[leaf] = best.feature;
      }
    }
  }
  __syncthreads();
  if (warp != 0) return;
  __threadfence_block();
  // split_info.rs:125-133 — first arg-max leaf under better_than.
  int bl = -1, bf = 0;
  double bg = 0.0;
  for (int i = lane; i < p.num_leaves; i += 32) {
    double g = J.bgain[i];
    int32_t fe = J.bfeat[i];
    if (bl < 0 || better_than(g, fe, bg, bf)) {
      bl = i;
      bg = g;
      bf = fe;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int oi = __shfl_xor_sync(FULL, bl, o);
    double og = __shfl_xor_sync(FULL, bg, o);
    int of = __shfl_xor_sync(FULL, bf, o);
    if (oi >= 0) {
      if (bl < 0 || better_than(og, of, bg, bf) || (!better_than(bg, bf, og, of) && oi < bl)) {
        bl = oi;
        bg = og;
        bf = of;
      }
    }
  }
  const Cand info = J.best[bl];
  if ((!(info.gain > 0.0) && !isnan(info.gain)) || info.inner < 0) {  // serial.rs:611 — gain <= 0 stops
    if (lane == 0) st->stop = 1;
    return;
  }
  const DevFeature m = feats[info.inner];
  for (int b = lane; b < 256; b += 32)
    st->route[b] = b < m.gbins ? route_bin(m, info.threshold, info.default_left != 0, (uint32_t)b) : 0;
  if (lane == 0) {
    st->split_leaf = bl;
    st->split_inner = info.inner;
    st->new_leaf = st->tree_leaves;
  }
}

// Root of a tree (serial.rs:658-776 after the root sums, then :580-586 and the first
// BeforeFindBestSplit). leaf_sum[0] and root_count are already set.
__global__ void __launch_bounds__(256) k_tree_begin(const Job* __restrict__ jobs, Params p) {
  const Job& J = jobs[blockIdx.z];
  JobState* st = J.st;
  for (int i = threadIdx.x; i < p.num_leaves; i += blockDim.x) {
    J.leaf_begin[i] = 0;
    J.leaf_count[i] = i == 0 ? st->root_count : 0;
    J.leaf_buf[i] = 0;
    J.leaf_depth[i] = 0;
    J.leaf_slot[i] = -1;
    J.leaf_value[i] = 0.0;
    Cand c;
    cand_reset(&c, -1, -1);
    J.best[i] = c;
    J.bgain[i] = c.gain;
    J.bfeat[i] = -1;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lane == 0) {
      st->stop = 0;
      st->tree_leaves = 1;
      st->next_free = 0;
      const LeafSum r = J.leaf_sum[0];
      double root = leaf_output_root(p, r.sg, r.sh, r.num_data);
      st->root_output = round_to_zero(root);
      J.leaf_value[0] = st->root_output;
    }
    __syncwarp();
    before_find_best_split(J, p, st, 0, -1, lane);
  }
}

}  // namespace

void launch_search(const Job* d_jobs, int num_jobs, const Params& p, const DevFeature* feats, cudaStream_t s) {
  dim3 grid((unsigned)ceil_div64(2 * p.F, 2), 1, num_jobs);
  const bool plain = !p.use_l1 && !p.use_max && !p.use_smooth;
  if (p.quant) {
    if (plain) k_search<true, true><<<grid, 64, 0, s>>>(d_jobs, p, feats);
    else k_search<false, true><<<grid, 64, 0, s>>>(d_jobs, p, feats);
  } else {
    if (plain) k_search<true, false><<<grid, 64, 0, s>>>(d_jobs, p, feats);
    else k_search<false, false><<<grid, 64, 0, s>>>(d_jobs, p, feats);
  }
}


void launch_tree_begin(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s) {
  k_tree_begin<<<dim3(1, 1, num_jobs), 256, 0, s>>>(d_jobs, p);
}

}  // namespace bk

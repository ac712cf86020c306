// FindBestSplitsFromHistograms (serial.rs:1322-1566, int: :1212-1300) and the grow-loop
// bookkeeping kernels (serial.rs:578-628, :779-825, :1685-1876), GB300 form.
//
// k_search: one warp per feature. It fixes the smaller leaf's most-frequent bin
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
// k_decide: folds the per-feature candidates of each searched leaf in feature order with
// `better_than`, takes the arg-max leaf (split_info.rs:88-96), stops the tree when its gain is
// <= 0, and builds the route table of the chosen split (data_partition.rs:299-410).
// k_post_split: applies the partition result to the leaf records and prepares the next
// iteration (BeforeFindBestSplit), all on the device.
#include <math_constants.h>

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

// FindBestThresholdSequentially (float), feature_histogram.rs:363-663.
template <bool REV>
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
      // left starts as everything outside the slice (the most-frequent bin 0 and nothing else)
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
    // REV: p* are the right side; FWD: the left side.
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
    double gain = valid ? split_gains(p, slg, slh, srg, srh, lc, rc, parent) : -CUDART_INF;
    bool pass = valid && !(gain <= mgs);
    if (__any_sync(FULL, pass)) r.splittable = 1;
    double bg;
    int bl = warp_best_lane(pass && gain > r.gain, gain, lane, &bg);
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

// FindBestThresholdSequentiallyInt, feature_histogram.rs:839-1142.
template <bool REV>
__device__ DirBest scan_int(const Params& p, const DevFeature& m, const IntHist& H, bool SKIP, bool NA, int64_t tg,
                            int64_t th, double gs, double hs, int32_t num_data, double mgs, double parent, int lane) {
  DirBest r;
  r.splittable = 0;
  r.gain = -CUDART_INF;
  r.th = m.num_bin;
  r.lc = 0;
  r.slg = r.slh = 0.0;
  r.lg = r.lh = 0;
  const double cnt_factor = (double)num_data / (double)th;
  const int off = m.offset;
  int64_t cg, ch;
  int t_first, P;
  if (REV) {
    t_first = m.num_bin - 1 - off - (NA ? 1 : 0);
    P = t_first - (1 - off) + 1;
    cg = ch = 0;
  } else {
    int t_end = m.num_bin - 2 - off;
    if (NA && off == 1) {
      int64_t pg = 0, ph = 0;
      for (int i = lane; i < m.num_bin - off; i += 32) {
        int64_t v = H.get(i);
        pg += unpack_g(v);
        ph += unpack_h(v);
      }
      cg = tg - warp_sum(pg);
      ch = th - warp_sum(ph);
      t_first = -1;
    } else {
      cg = ch = 0;
      t_first = 0;
    }
    P = t_end - t_first + 1;
  }
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
    bool first, brk;
    int64_t lg, lh, rg, rh;
    int32_t lc, rc;
    double slh, srh;
    if (REV) {
      rg = pg;
      rh = ph;
      rc = round_int((double)rh * cnt_factor);
      srh = (double)rh * hs;
      first = cand && !(rc < p.min_data || srh < p.min_hess);
      lc = num_data - rc;
      lh = th - rh;
      slh = (double)lh * hs;
      brk = first && (lc < p.min_data || slh < p.min_hess);
      lg = tg - rg;
    } else {
      lg = pg;
      lh = ph;
      lc = round_int((double)lh * cnt_factor);
      slh = (double)lh * hs;
      first = cand && !(lc < p.min_data || slh < p.min_hess);
      rc = num_data - lc;
      rh = th - lh;
      srh = (double)rh * hs;
      brk = first && (rc < p.min_data || srh < p.min_hess);
      rg = tg - lg;
    }
    unsigned bm = __ballot_sync(FULL, brk);
    int stop_lane = bm ? __ffs(bm) - 1 : 32;
    bool valid = first && !brk && lane < stop_lane;
    double gain = -CUDART_INF;
    if (valid) {
      double slg = (double)lg * gs;
      double srg = (double)rg * gs;
      gain = split_gains(p, slg, slh + BK_EPS, srg, srh + BK_EPS, lc, rc, parent);
    }
    bool pass = valid && !(gain <= mgs);
    if (__any_sync(FULL, pass)) r.splittable = 1;
    double bg;
    int bl = warp_best_lane(pass && gain > r.gain, gain, lane, &bg);
    if (bl < 32) {
      r.gain = bg;
      r.th = __shfl_sync(FULL, REV ? (t - 1 + off) : (t + off), bl);
      r.lg = __shfl_sync(FULL, lg, bl);
      r.lh = __shfl_sync(FULL, lh, bl);
    }
    if (bm) break;
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
__device__ void search_leaf_float(const Params& p, const DevFeature& m, const FloatHist& H, const LeafSum& ls,
                                  double parent, int lane, Cand* out, int32_t f) {
  const double sum_g = ls.sg;
  const double sum_h = ls.sh + 2.0 * BK_EPS;
  const int32_t num_data = ls.num_data;
  double gain_shift = leaf_gain(p, sum_g, sum_h, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  DirBest d[2];
  int nd;
  bool rev_of[2];
  if (m.num_bin > 2 && m.missing != 0) {
    bool skip = m.missing == 1, na = m.missing == 2;
    d[0] = scan_float<true>(p, m, H, skip, na, sum_g, sum_h, num_data, mgs, parent, lane);
    d[1] = scan_float<false>(p, m, H, skip, na, sum_g, sum_h, num_data, mgs, parent, lane);
    nd = 2;
  } else {
    d[0] = scan_float<true>(p, m, H, false, false, sum_g, sum_h, num_data, mgs, parent, lane);
    nd = 1;
  }
  rev_of[0] = true;
  rev_of[1] = false;
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
      c.default_left = rev_of[i] ? 1 : 0;
    }
  }
  if (nd == 1 && m.missing == 2) c.default_left = 0;
  c.gain *= m.penalty;
  c.splittable = sp;
  *out = c;
}

// FindBestThresholdInt for one leaf: feature_histogram.rs:673-830.
__device__ void search_leaf_int(const Params& p, const DevFeature& m, const IntHist& H, const LeafSum& ls,
                                double gs, double hs, double parent, int lane, Cand* out, int32_t f) {
  const int64_t tg = ls.int_sum >> 32;
  const int64_t th = ls.int_sum & 0xffffffffLL;
  const int32_t num_data = ls.num_data;
  const double sum_g = (double)tg * gs;
  const double sum_h = (double)th * hs;
  double gain_shift = leaf_gain(p, sum_g, sum_h, num_data, parent);
  double mgs = gain_shift + p.min_gain;
  DirBest d[2];
  int nd;
  if (m.num_bin > 2 && m.missing != 0) {
    bool skip = m.missing == 1, na = m.missing == 2;
    d[0] = scan_int<true>(p, m, H, skip, na, tg, th, gs, hs, num_data, mgs, parent, lane);
    d[1] = scan_int<false>(p, m, H, skip, na, tg, th, gs, hs, num_data, mgs, parent, lane);
    nd = 2;
  } else {
    d[0] = scan_int<true>(p, m, H, false, false, tg, th, gs, hs, num_data, mgs, parent, lane);
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
}

__device__ __forceinline__ double parent_output_of(const Params& p, const JobState* st, const LeafSum& ls) {
  // serial.rs:1924-1935 (GetParentOutput)
  if (st->tree_leaves == 1) return leaf_output_root(p, ls.sg, ls.sh, ls.num_data);
  return ls.weight;
}

__global__ void __launch_bounds__(128) k_search(const Job* __restrict__ jobs, Params p,
                                                const DevFeature* __restrict__ feats) {
  const Job& J = jobs[blockIdx.z];
  const JobState* st = J.st;
  if (st->stop || !st->do_search) return;
  const int lane = threadIdx.x & 31;
  const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (f >= p.F) return;
  if (!J.used[f]) return;
  const DevFeature m = feats[f];
  const int tile = f / TILE, fl = f % TILE;
  const size_t slot_stride = (size_t)p.T * p.B * TILE;
  const size_t feat_off = (size_t)tile * p.B * TILE + fl;
  const int32_t sl = st->smaller_leaf, ll = st->larger_leaf;
  const LeafSum S = J.leaf_sum[sl];
  const double sp_out = parent_output_of(p, st, S);
  if (p.quant) {
    int64_t* pool = reinterpret_cast<int64_t*>(J.pool);
    IntHist HS{pool + (size_t)st->smaller_slot * slot_stride + feat_off};
    // FixHistogram on the smaller leaf (exact integers)
    if (m.mfb > 0) {
      int64_t acc = 0;
      for (int i = lane; i < m.num_bin; i += 32)
        if (i != m.mfb) acc += HS.get(i);
      acc = warp_sum(acc);
      // the packed leaf total (grad << 32) | hess equals grad * 2^32 + hess, so packed
      // arithmetic is exact componentwise
      if (lane == 0) HS.base[(size_t)(m.mfb + 1) * TILE] = S.int_sum - acc;
      __syncwarp();
    }
    if (ll >= 0) {
      IntHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
      for (int i = lane; i < m.len; i += 32) HL.base[(size_t)(i + 1) * TILE] -= HS.get(i);
      __syncwarp();
    }
    const double gs = st->gscale, hs = st->hscale;
    search_leaf_int(p, m, HS, S, gs, hs, sp_out, lane, &J.cand[f], f);
    if (ll >= 0) {
      IntHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
      const LeafSum Lg = J.leaf_sum[ll];
      double lp_out = parent_output_of(p, st, Lg);
      search_leaf_int(p, m, HL, Lg, gs, hs, lp_out, lane, &J.cand[p.F + f], f);
    }
  } else {
    double2* pool = reinterpret_cast<double2*>(J.pool);
    FloatHist HS{pool + (size_t)st->smaller_slot * slot_stride + feat_off};
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
      if (lane == 0) HS.base[(size_t)(m.mfb + 1) * TILE] = make_double2(S.sg - ag, S.sh - ah);
      __syncwarp();
    }
    if (ll >= 0) {
      FloatHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
      for (int i = lane; i < m.len; i += 32) {
        double2 a = HL.get(i), b = HS.get(i);
        HL.base[(size_t)(i + 1) * TILE] = make_double2(a.x - b.x, a.y - b.y);
      }
      __syncwarp();
    }
    search_leaf_float(p, m, HS, S, sp_out, lane, &J.cand[f], f);
    if (ll >= 0) {
      FloatHist HL{pool + (size_t)st->larger_slot * slot_stride + feat_off};
      const LeafSum Lg = J.leaf_sum[ll];
      double lp_out = parent_output_of(p, st, Lg);
      search_leaf_float(p, m, HL, Lg, lp_out, lane, &J.cand[p.F + f], f);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// k_decide
// ---------------------------------------------------------------------------------------------

// The route of one stored bin for a numerical split of a single-feature dense group
// (data_partition.rs:299-410 with group_view :25-40: min_bin 1, max_bin gbins - 1,
// use_min_bin false). 1 = left.
__device__ uint8_t route_bin(const DevFeature& m, uint32_t threshold, bool default_left, uint32_t bin) {
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

__device__ __forceinline__ bool cand_better(const Cand& a, const Cand& b) {
  return better_than(a.gain, a.feature, b.gain, b.feature);
}

__global__ void __launch_bounds__(64) k_decide(const Job* __restrict__ jobs, Params p,
                                               const DevFeature* __restrict__ feats) {
  const Job& J = jobs[blockIdx.z];
  JobState* st = J.st;
  if (st->stop) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (st->do_search) {
    // serial.rs:1523-1558 — fold the candidates of each searched leaf in feature order.
    const int32_t leaf = warp == 0 ? st->smaller_leaf : st->larger_leaf;
    const int32_t slot = warp == 0 ? st->smaller_slot : st->larger_slot;
    if (leaf >= 0) {
      int bf = -1;  // best feature index among this lane's features (NaN gains never win)
      for (int f = lane; f < p.F; f += 32) {
        if (!J.used[f]) continue;
        const Cand& c = J.cand[warp * p.F + f];
        J.splittable[(size_t)slot * p.F + f] = (uint8_t)c.splittable;
        if (isnan(c.gain)) continue;
        if (bf < 0 || cand_better(c, J.cand[warp * p.F + bf])) bf = f;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        int of = __shfl_xor_sync(FULL, bf, o);
        if (of >= 0 && (bf < 0 || cand_better(J.cand[warp * p.F + of], J.cand[warp * p.F + bf]))) bf = of;
      }
      if (lane == 0) {
        Cand best;
        cand_reset(&best, -1, -1);
        // The reference starts from SplitInfo::default (gain -inf, feature -1) and replaces it
        // only with a better candidate.
        if (bf >= 0 && cand_better(J.cand[warp * p.F + bf], best)) best = J.cand[warp * p.F + bf];
        J.best[leaf] = best;
      }
    }
  }
  __syncthreads();
  if (warp != 0) return;
  // split_info.rs:125-133 — first arg-max leaf under better_than.
  int bl = -1;
  for (int i = lane; i < p.num_leaves; i += 32) {
    if (bl < 0 || cand_better(J.best[i], J.best[bl])) bl = i;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int ob = __shfl_xor_sync(FULL, bl, o);
    if (ob >= 0) {
      if (bl < 0) bl = ob;
      else if (cand_better(J.best[ob], J.best[bl])) bl = ob;
      else if (!cand_better(J.best[bl], J.best[ob]) && ob < bl) bl = ob;
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

// ---------------------------------------------------------------------------------------------
// k_post_split: serial.rs:1685-1876 after the partition, then :779-825 for the next iteration.
// ---------------------------------------------------------------------------------------------
__device__ void before_find_best_split(const Job& J, const Params& p, JobState* st, int32_t left, int32_t right,
                                       int lane) {
  bool go = true;
  if (p.max_depth > 0 && J.leaf_depth[left] >= p.max_depth) go = false;
  int32_t nl = (int32_t)J.leaf_count[left];
  int32_t nr = right >= 0 ? (int32_t)J.leaf_count[right] : 0;
  if (go && nr < p.min_data * 2 && nl < p.min_data * 2) go = false;
  if (!go) {
    if (lane == 0) {
      J.best[left].gain = -CUDART_INF;
      if (right >= 0) J.best[right].gain = -CUDART_INF;
      st->do_search = 0;
    }
    return;
  }
  int32_t smaller_slot, parent_slot;
  if (right < 0) {
    smaller_slot = st->next_free;
    parent_slot = -1;
    if (lane == 0) {
      st->next_free += 1;
      J.leaf_slot[left] = smaller_slot;
      st->smaller_leaf = left;
      st->larger_leaf = -1;
      st->smaller_slot = smaller_slot;
      st->larger_slot = -1;
      st->parent_slot = -1;
      st->use_subtract = 0;
    }
  } else {
    parent_slot = J.leaf_slot[left];
    smaller_slot = st->next_free;
    if (lane == 0) {
      st->next_free += 1;
      if (nl < nr) {  // the left child is smaller: the right child inherits the parent's slot
        J.leaf_slot[right] = parent_slot;
        J.leaf_slot[left] = smaller_slot;
        st->smaller_leaf = left;
        st->larger_leaf = right;
      } else {
        J.leaf_slot[right] = smaller_slot;
        st->smaller_leaf = right;
        st->larger_leaf = left;
      }
      st->smaller_slot = smaller_slot;
      st->larger_slot = parent_slot;
      st->parent_slot = parent_slot;
      st->use_subtract = 1;
    }
  }
  if (lane == 0) {
    int32_t sl = right < 0 ? left : (nl < nr ? left : right);
    int64_t rows = J.leaf_count[sl];
    if (rows == p.n) st->hist_rows_direct += rows;
    else st->hist_rows_gather += rows;
    st->hist_builds += 1;
  }
  // serial.rs:840-854 — features the parent could not split are skipped for both children.
  for (int f = lane; f < p.F; f += 32) {
    uint8_t u = parent_slot < 0 ? 1 : J.splittable[(size_t)parent_slot * p.F + f];
    J.used[f] = u;
    if (!u) J.splittable[(size_t)smaller_slot * p.F + f] = 0;
  }
  if (lane == 0) st->do_search = 1;
}

__global__ void __launch_bounds__(32) k_post_split(const Job* __restrict__ jobs, Params p,
                                                   const DevFeature* __restrict__ feats) {
  const Job& J = jobs[blockIdx.z];
  JobState* st = J.st;
  if (st->stop) return;
  const int lane = threadIdx.x;
  const int32_t bl = st->split_leaf, nl = st->new_leaf;
  const int64_t L = st->total_left;
  const int64_t b = J.leaf_begin[bl], c = J.leaf_count[bl];
  const int32_t buf = J.leaf_buf[bl];
  Cand info = J.best[bl];
  __syncwarp();
  if (lane == 0) {
    J.leaf_count[bl] = L;
    J.leaf_begin[nl] = b + L;
    J.leaf_count[nl] = c - L;
    J.leaf_buf[bl] = 1 - buf;
    J.leaf_buf[nl] = 1 - buf;
    info.left_count = (int32_t)L;
    info.right_count = (int32_t)(c - L);
    bk_split& r = J.records[st->tree_leaves - 1];
    r.leaf = bl;
    r.right_leaf = nl;
    r.inner_feature = info.inner;
    r.real_feature = info.feature;
    r.threshold = info.threshold;
    r.default_left = info.default_left;
    r.missing_type = feats[info.inner].missing;
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
    J.leaf_value[bl] = isnan(info.left_output) ? 0.0 : info.left_output;
    J.leaf_value[nl] = isnan(info.right_output) ? 0.0 : info.right_output;
    J.leaf_depth[nl] = J.leaf_depth[bl] + 1;
    J.leaf_depth[bl] += 1;
    LeafSum ls{info.lsg, info.lsh, info.left_output, info.lint, info.left_count, 0};
    LeafSum rs{info.rsg, info.rsh, info.right_output, info.rint, info.right_count, 0};
    J.leaf_sum[bl] = ls;
    J.leaf_sum[nl] = rs;
    J.best[bl] = info;
    st->tree_leaves += 1;
  }
  __syncwarp();
  before_find_best_split(J, p, st, bl, nl, lane);
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
  dim3 grid((unsigned)ceil_div64(p.F, 4), 1, num_jobs);
  k_search<<<grid, 128, 0, s>>>(d_jobs, p, feats);
}

void launch_decide(const Job* d_jobs, int num_jobs, const Params& p, const DevFeature* feats, cudaStream_t s) {
  k_decide<<<dim3(1, 1, num_jobs), 64, 0, s>>>(d_jobs, p, feats);
}

void launch_post_split(const Job* d_jobs, int num_jobs, const Params& p, const DevFeature* feats, cudaStream_t s) {
  k_post_split<<<dim3(1, 1, num_jobs), 32, 0, s>>>(d_jobs, p, feats);
}

void launch_tree_begin(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s) {
  k_tree_begin<<<dim3(1, 1, num_jobs), 256, 0, s>>>(d_jobs, p);
}

}  // namespace bk

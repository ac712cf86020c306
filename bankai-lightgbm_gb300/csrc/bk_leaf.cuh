// Per-leaf constants of a split search: the preamble of FindBestThreshold / FindBestThresholdInt
// (feature_histogram.rs:219-240, :673-700) that every feature of a leaf shares — the leaf's sums,
// its parent output (serial.rs:1924-1935), min_gain_shift, the count factor and, on the quantized
// path, the integer validity thresholds of the threshold scans. They are computed once per search
// by one CTA of the histogram launch that precedes it, so the search warps start from them.
#pragma once
#include "bk_common.cuh"
#include "bk_grow.cuh"
#include "bk_math.cuh"

namespace bk {

// Smallest x in [0, hi) with pred(x) (monotone false -> true), or hi; one warp, 32-ary search.
template <typename Pred>
__device__ int64_t warp_first_true(int64_t hi, int lane, Pred pred) {
  int64_t lo = 0;
  while (lo < hi) {
    int64_t step = (hi - lo + 31) >> 5;  // hi > lo: a shift, not an int64 division
    int64_t x = lo + (int64_t)lane * step;
    bool t = x < hi && pred(x);
    unsigned m = __ballot_sync(0xffffffffu, t);
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

// As warp_first_true, trying first the 32 values around `guess` (one warp-wide evaluation) and
// falling back to the full search when the answer lies outside that window.
template <typename Pred>
__device__ int64_t warp_first_true_near(int64_t hi, int64_t guess, int lane, Pred pred) {
  guess = guess < 0 ? 0 : (guess > hi ? hi : guess);
  const int64_t x = guess - 15 + lane;
  const bool t = x >= hi ? true : (x < 0 ? false : pred(x));
  const unsigned m = __ballot_sync(0xffffffffu, t);
  if (m != 0u && (m & 1u) == 0u) return guess - 15 + (__ffs(m) - 1);  // false -> true inside
  if (m != 0u && guess - 15 <= 0) return 0;  // everything from 0 on is true
  return warp_first_true(hi, lane, pred);
}

// Integer thresholds of a leaf (feature-independent): for an accumulated side with integer hessian
// x, the reference's `count >= min_data && hess >= min_hessian` test (counts estimated as
// round_int(x * cnt_factor), feature_histogram.rs:927-940) is monotone in x, so it is x >= first_x;
// and the `break` test on the other side is x >= brk_x.
__device__ __forceinline__ void int_thresholds(const Params& p, int64_t th, double hs, int32_t num_data, int lane,
                                               int64_t* first_x, int64_t* brk_x) {
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
  *first_x = cnt_ok > hess_ok ? cnt_ok : hess_ok;
  int64_t hess_brk = th - hess_ok + 1;  // (th - x) * hs < min_hess  <=>  th - x < hess_ok
  *brk_x = cnt_brk < hess_brk ? cnt_brk : hess_brk;
}

__device__ __forceinline__ double parent_output_of(const Params& p, bool root, const LeafSum& ls) {
  // serial.rs:1924-1935 (GetParentOutput)
  if (root) return leaf_output_root(p, ls.sg, ls.sh, ls.num_data);
  return ls.weight;
}

// One warp: the constants of side `side` (0 = smaller leaf, 1 = larger leaf) of the coming search,
// for a leaf with sums `ls` (`root`: the tree's only leaf).
__device__ __forceinline__ void compute_leaf_const_ls(const Job& J, const Params& p, const JobState* st, int side,
                                                      const LeafSum& ls, bool root, int lane) {
  LeafConst c;
  c.first_x = c.brk_x = 0;
  if (p.quant) {
    const int64_t tg = ls.int_sum >> 32, th = ls.int_sum & 0xffffffffLL;
    c.sum_g = (double)tg * st->gscale;
    c.sum_h = (double)th * st->hscale;
    c.cnt_factor = (double)ls.num_data / (double)th;
    int_thresholds(p, th, st->hscale, ls.num_data, lane, &c.first_x, &c.brk_x);
  } else {
    c.sum_g = ls.sg;
    c.sum_h = ls.sh + 2.0 * BK_EPS;
    c.cnt_factor = (double)ls.num_data / c.sum_h;
  }
  c.parent = parent_output_of(p, root, ls);
  c.mgs = leaf_gain(p, c.sum_g, c.sum_h, ls.num_data, c.parent) + p.min_gain;
  c.mgs_up = __double2float_ru(c.mgs);
  c.mgs_dn = __double2float_rd(c.mgs);
  c.gsf = (float)st->gscale;
  c.hsf = (float)st->hscale;
  c.l2f = (float)p.l2;
  c._pad = 0.f;
  c.gs = st->gscale;
  c.hs = st->hscale;
  c.ls = ls;
  if (lane == 0) J.lconst[side] = c;
}

__device__ __forceinline__ void compute_leaf_const(const Job& J, const Params& p, const JobState* st, int side,
                                                   int lane) {
  const int32_t leaf = side ? st->larger_leaf : st->smaller_leaf;
  if (leaf < 0) return;
  compute_leaf_const_ls(J, p, st, side, J.leaf_sum[leaf], st->tree_leaves == 1, lane);
}

// ColSampler::get_by_node (col_sampler.rs:109-177) for side `side` of the coming search, on one
// thread. With interaction constraints the allowed features are the leaf's path features plus
// every constraint set that holds the whole path (every set at the root); `extra` is a feature
// the path gains with the split being applied (-1: none). Without sampling the mask is the
// allowed set; with sampling it is Random::sample (utils/random.rs:53-80) of get_cnt(n, fraction)
// positions (at most the allowed candidates) among the candidates — the tree's by-tree sample
// (ascending inner features) when one is active, else every feature — filtered by the allowed
// set, continuing the sampler's LCG stream kept in the job state.
__device__ __forceinline__ uint32_t lcg_step(uint32_t x) { return x * 214013u + 2531011u; }

__device__ __forceinline__ bool path_has(const uint32_t* path, int f, int extra) {
  return f == extra || ((path[f >> 5] >> (f & 31)) & 1u) != 0u;
}

__device__ __forceinline__ void draw_node_sample(const Job& J, const Params& p, JobState* st, int side, int32_t leaf,
                                                 int extra) {
  uint8_t* out = J.used + (size_t)(1 + side) * p.F;
  uint8_t* sel = J.used + (size_t)3 * p.F;
  const bool bytree = st->bytree_on != 0;
  const bool constrained = p.n_icons > 0;
  const bool sampled = st->bynode_fraction < 1.0;
  // the allowed features
  if (!constrained) {
    for (int f = 0; f < p.F; ++f) out[f] = 1;
  } else {
    const uint32_t* path = leaf_path_bits(J, p, leaf);
    bool empty = extra < 0;
    for (int w = 0; w < p.path_words && empty; ++w) empty = path[w] == 0u;
    for (int f = 0; f < p.F; ++f) out[f] = path_has(path, f, extra) ? 1 : 0;
    for (int c = 0; c < p.n_icons; ++c) {
      const uint32_t* set = p.icons + (size_t)c * p.path_words;
      bool holds = true;  // every path feature is in the set
      for (int f = 0; f < p.F && holds && !empty; ++f)
        if (path_has(path, f, extra) && ((set[f >> 5] >> (f & 31)) & 1u) == 0u) holds = false;
      if (empty || holds)
        for (int f = 0; f < p.F; ++f) out[f] |= (uint8_t)((set[f >> 5] >> (f & 31)) & 1u);
    }
  }
  if (!sampled) return;
  int32_t n_all = 0, n = 0;
  for (int f = 0; f < p.F; ++f) {
    const bool cand = !bytree || J.tree_mask[f];
    n_all += cand ? 1 : 0;
    n += (cand && out[f]) ? 1 : 0;
    sel[f] = 0;
  }
  const int32_t used = (int32_t)((double)n_all * st->bynode_fraction + 0.5);
  const int32_t mn = n_all < 1 ? n_all : 1;
  int32_t k = used > mn ? used : mn;
  if (constrained && n < k) k = n;
  uint32_t x = st->col_rng;
  if (k > n || k <= 0) {
    // no position is drawn
  } else if (k == n) {
    for (int32_t q = 0; q < n; ++q) sel[q] = 1;
  } else if (k > 1 && (double)k > (double)n / ((k & (k - 1)) == 0 ? (double)(31 - __clz(k)) : log2((double)k))) {
    int32_t got = 0;
    for (int32_t i = 0; i < n; ++i) {
      x = lcg_step(x);
      const float r = (float)((x >> 16) & 0x7fffu) / 32768.0f;
      const double prob = (double)(k - got) / (double)(n - i);
      if ((double)r < prob) {
        sel[i] = 1;
        ++got;
      }
    }
  } else {
    for (int32_t r = n - k; r < n; ++r) {
      x = lcg_step(x);
      const int32_t v = (int32_t)(x & 0x7fffffffu) % (r + 1);
      if (sel[v]) sel[r] = 1;
      else sel[v] = 1;
    }
  }
  st->col_rng = x;
  for (int32_t f = 0, q = 0; f < p.F; ++f) {
    const bool cand = (!bytree || J.tree_mask[f]) && out[f];
    out[f] = cand ? sel[q++] : 0;
  }
}

// The by-node masks of a search: the smaller leaf's, then the larger leaf's, if any
// (serial.rs:1328-1336). `small` / `large` name the leaves whose paths the masks use.
__device__ __forceinline__ void draw_node_samples(const Job& J, const Params& p, int32_t small, int32_t large,
                                                  int extra) {
  JobState* st = J.st;
  draw_node_sample(J, p, st, 0, small, extra);
  if (large >= 0) draw_node_sample(J, p, st, 1, large, extra);
}

// The histogram CTA that does the serial side work of its launch: the last CTA of tile 0, idle for
// leaves that do not need the whole grid.
__device__ __forceinline__ bool hist_side_cta() { return blockIdx.x == gridDim.x - 1 && blockIdx.y == 0; }

// Called by every thread of a histogram CTA before its row loop: the side CTA computes both sides'
// constants with its first two warps, from the leaf records.
__device__ __forceinline__ void hist_leaf_constants(const Job& J, const Params& p) {
  if (!hist_side_cta() || threadIdx.x >= 128) return;
  const JobState* st = J.st;
  if (st->stop || !st->do_search) return;
  if (threadIdx.x >= 64) {
    if (p.bynode && threadIdx.x == 96) draw_node_samples(J, p, st->smaller_leaf, st->larger_leaf, -1);
    return;
  }
  compute_leaf_const(J, p, st, (int)(threadIdx.x >> 5), (int)(threadIdx.x & 31));
}

// The same when the launch also applies the previous split (the single-pass partition leaves it
// to the histogram launch): the side CTA's warps 0 / 1 compute the constants from the split's
// candidate record and row counts, warp 2 writes the split's bookkeeping.
__device__ __forceinline__ void hist_apply_split(const Job& J, const Params& p, const SplitOutcome& o) {
  if (!hist_side_cta() || threadIdx.x >= 128) return;
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  if (warp == 2) {
    post_split_writes(J, p, o, lane);
    return;
  }
  if (!o.go) return;
  if (warp == 3) {
    // both children's paths are the split leaf's plus the split feature (warp 2 is writing them
    // now; either value of the split leaf's path, with that feature added, is the children's)
    if (p.bynode && lane == 0) draw_node_samples(J, p, o.bl, o.bl, J.st->split_inner);
    return;
  }
  const JobState* st = J.st;
  const Cand& info = J.cand[(size_t)o.bl * p.F + st->split_inner];
  LeafSum small, large;
  split_children(info, o, &small, &large);
  compute_leaf_const_ls(J, p, st, warp, warp ? large : small, false, lane);
}

}  // namespace bk

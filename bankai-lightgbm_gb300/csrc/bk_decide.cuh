// The split decision after a search (serial.rs:1523-1558 fold of each searched leaf's candidates
// in feature order, split_info.rs:67-133 better_than / argmax over the leaves, serial.rs:611 stop
// on a gain <= 0): shared by the search launch (its last CTA decides) and the single-pass
// partition (every CTA decides the same split from the same records, CTA 0 records it).
#pragma once
#include <math_constants.h>

#include "bk_common.cuh"

namespace bk {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kDecideThreads = 256;  // the decision runs on one 256-thread CTA
constexpr int kDecideWarps = kDecideThreads / 32;
constexpr long long kNoKey = (long long)0x8000000000000000ULL;

// Order-preserving integer key of an f64 gain (the fold and arg-max compare keys, not doubles:
// f64 comparisons are slow on this part).
__device__ __forceinline__ long long dkey(double x) {
  long long b = __double_as_longlong(x);
  if (b == kNoKey) b = 0;
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dnan(double x) {
  return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL) > 0x7ff0000000000000ULL;
}


// split_info.rs:104-121 (better_than) on keys: the higher gain, then the smaller real feature
// (-1 counts as largest); with a NaN gain on either side neither is better.
__device__ __forceinline__ bool better_k(long long ka, bool na, int fa, long long kb, bool nb, int fb) {
  if (na || nb) return false;
  if (ka != kb) return ka > kb;
  const int a = fa == -1 ? 0x7fffffff : fa;
  const int b = fb == -1 ? 0x7fffffff : fb;
  return a < b;
}

struct Pick {
  int i, f;     // index (-1: none), real feature
  long long k;  // dkey of the gain
  bool nan;
  double g;     // the gain
  long long pay;  // fold: threshold | default_left << 31; leaf arg-max: the split descriptor
};

// Fold step: `a` comes first in the sequential order; `b` replaces it only when strictly better;
// NaN gains never win (the sequential fold never adopts them).
__device__ __forceinline__ void pick(Pick& a, const Pick& b) {
  if (b.i < 0 || b.nan) return;
  if (a.i < 0 || better_k(b.k, false, b.f, a.k, a.nan, a.f) || (!better_k(a.k, a.nan, a.f, b.k, false, b.f) && b.i < a.i))
    a = b;
}

// Arg-max step over leaves: the first arg-max under better_than, ties to the smaller index.
__device__ __forceinline__ void leaf_pick(Pick& a, const Pick& b) {
  if (b.i < 0) return;
  if (a.i < 0 || better_k(b.k, b.nan, b.f, a.k, a.nan, a.f) || (!better_k(a.k, a.nan, a.f, b.k, b.nan, b.f) && b.i < a.i))
    a = b;
}

__device__ __forceinline__ Pick shfl_pick(const Pick& a, int src_or_mask, bool xor_mode) {
  Pick b;
  if (xor_mode) {
    b.i = __shfl_xor_sync(FULL, a.i, src_or_mask);
    b.f = __shfl_xor_sync(FULL, a.f, src_or_mask);
    b.k = __shfl_xor_sync(FULL, a.k, src_or_mask);
    b.nan = __shfl_xor_sync(FULL, (int)a.nan, src_or_mask) != 0;
    b.g = __shfl_xor_sync(FULL, a.g, src_or_mask);
    b.pay = __shfl_xor_sync(FULL, a.pay, src_or_mask);
  } else {
    b.i = __shfl_sync(FULL, a.i, src_or_mask);
    b.f = __shfl_sync(FULL, a.f, src_or_mask);
    b.k = __shfl_sync(FULL, a.k, src_or_mask);
    b.nan = __shfl_sync(FULL, (int)a.nan, src_or_mask) != 0;
    b.g = __shfl_sync(FULL, a.g, src_or_mask);
    b.pay = __shfl_sync(FULL, a.pay, src_or_mask);
  }
  return b;
}

__device__ __forceinline__ long long warp_max64(long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long y = __shfl_xor_sync(FULL, x, o);
    x = y > x ? y : x;
  }
  return x;
}

// The warp's arg-max under pick / leaf_pick when no valid lane holds a NaN gain: the order is then
// total (higher key, then the smaller real feature with -1 last, then the smaller index), so a
// 64-bit max and two 32-bit min reductions replace the record-by-record tree of shuffles. Every
// lane gets the winner (index -1: no valid lane).
__device__ __forceinline__ Pick warp_argmax(const Pick& x, bool valid, int lane) {
  const long long km = warp_max64(valid ? x.k : kNoKey);
  if (km == kNoKey) {
    Pick n = x;
    n.i = -1;
    return n;
  }
  const bool at = valid && x.k == km;
  const int fa = x.f == -1 ? 0x7fffffff : x.f;
  const int fm = __reduce_min_sync(FULL, at ? fa : 0x7fffffff);
  const bool at2 = at && fa == fm;
  const int im = __reduce_min_sync(FULL, at2 ? x.i : 0x7fffffff);
  const int wl = __ffs(__ballot_sync(FULL, at2 && x.i == im)) - 1;
  (void)lane;
  return shfl_pick(x, wl, false);
}

__device__ __forceinline__ Pick make_pick(int i, double g, int f, long long pay) {
  return Pick{i, f, dkey(g), dnan(g), g, pay};
}

// The chosen split, as every CTA that decides it sees it.
struct Decision {
  int32_t stop, leaf, inner, buf, depth, sslot, new_leaf, pslot;
  uint32_t thr;  // threshold | default_left << 31
  int64_t begin, count;
};

// Shared memory of a split decision.
struct DecideSmem {
  Pick f[kDecideWarps], l[kDecideWarps];  // per warp: the fold's and the leaf arg-max's partials
  // the row range of the first kDecideThreads leaves, so the chosen leaf's is at hand for the
  // partition that follows
  int64_t lb[kDecideThreads], lc[kDecideThreads];
  int32_t lbuf[kDecideThreads], ld[kDecideThreads], lslot[kDecideThreads];
  int32_t stopped, searched, leaf0, leaf1;
  // the pool slots of the searched leaves, the next free slot and the leaf count (the histogram
  // launch's bookkeeping wrote them)
  int32_t slot0, slot1, next_free, tree_leaves;
};

// Part one of a split decision (split_info.rs:125-133): the arg-max over every leaf but the two
// the current search covers, whose records the histogram launch of this step and earlier steps
// wrote, and the loads of the job-state fields part two needs (the searched leaves' pool slots,
// the next free slot, the leaf count: the histogram launch's bookkeeping wrote them). A launch
// that follows the search can run it before its griddep_wait: the search triggers its dependents
// only after its own wait, so by then the histogram launch has completed; the loads go through L2
// (__ldcg). Every thread of the CTA calls it; no barrier.
__device__ __forceinline__ void decide_leaves(const Job& J, const Params& p, DecideSmem& ds) {
  const JobState* st = J.st;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const bool stopped = __ldcg(&st->stop) != 0;
  const bool searched = __ldcg(&st->do_search) != 0;
  const int32_t leaf0 = __ldcg(&st->smaller_leaf), leaf1 = __ldcg(&st->larger_leaf);
  if (t == 0) {
    ds.stopped = stopped;
    ds.searched = searched;
    ds.leaf0 = leaf0;
    ds.leaf1 = leaf1;
    ds.slot0 = __ldcg(&st->smaller_slot);
    ds.slot1 = __ldcg(&st->larger_slot);
    ds.next_free = __ldcg(&st->next_free);
    ds.tree_leaves = __ldcg(&st->tree_leaves);
  }
  Pick b{-1, 0, 0, false, 0.0, 0};
  for (int i = t; i < p.num_leaves; i += kDecideThreads) {
    if (i < kDecideThreads) {
      ds.lb[i] = __ldcg(&J.leaf_begin[i]);
      ds.lc[i] = __ldcg(&J.leaf_count[i]);
      ds.lbuf[i] = __ldcg(&J.leaf_buf[i]);
      ds.ld[i] = __ldcg(&J.leaf_depth[i]);
      ds.lslot[i] = __ldcg(&J.leaf_slot[i]);
    }
    const double bg = __ldcg(&J.bgain[i]);
    const int32_t bf = __ldcg(&J.bfeat[i]);
    const int64_t bs = __ldcg(&J.bsplit[i]);
    if (searched && (i == leaf0 || i == leaf1)) continue;
    leaf_pick(b, make_pick(i, bg, bf, bs));
  }
  if (__any_sync(FULL, b.i >= 0 && b.nan)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) leaf_pick(b, shfl_pick(b, o, true));
  } else {
    b = warp_argmax(b, b.i >= 0, lane);
  }
  if (lane == 0) ds.l[warp] = b;
}

// Part two (serial.rs:1523-1558, split_info.rs:125-133, serial.rs:611): the fold of the searched
// leaves' candidates in feature order (the first half of the CTA folds the smaller leaf, the second
// half the larger one), then the leaf arg-max over part one's partials and the searched leaves'
// new bests. Every thread gets the chosen split through `out` (written by thread 0: the caller
// synchronizes before reading it). With `record`, the decision's effects are written to the job:
// the searched leaves' new bests and splittable flags, the chosen split (the row range, depth and
// new pool slot the partition and the next histogram launch use) or the stop flag; without it
// nothing is written, so several CTAs can decide the same split from the same records. Candidates
// written by other CTAs are read through L2 (__ldcg). A leaf's best split stays in
// cand[leaf][feature]; the partition builds the route table of the chosen split from (inner,
// thr). A stopped tree gives out->stop = 1 and writes nothing. Call after decide_leaves and a
// barrier.
__device__ void decide_finish(const Job& J, const Params& p, const DevFeature* feats, bool record, Decision* out,
                              DecideSmem& ds) {
  JobState* st = J.st;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  constexpr int kHalf = kDecideThreads / 2;
  const bool stopped = ds.stopped != 0, searched = ds.searched != 0;
  const int32_t leaf0 = ds.leaf0, leaf1 = ds.leaf1;
  const Pick none{-1, 0x7fffffff, 0, false, 0.0, 0};
  Pick a = none;
  {
    const int side = t / kHalf;
    const int32_t leaf = side ? leaf1 : leaf0;
    const int32_t slot = side ? ds.slot1 : ds.slot0;
    for (int f = t % kHalf; f < p.F; f += kHalf) {
      const uint8_t u = J.used[f];
      const uint8_t cs = __ldcg(&J.csplit[side * p.F + f]);
      const double g = __ldcg(&J.cgain[side * p.F + f]);
      const uint32_t th = __ldcg(&J.cthr[side * p.F + f]);
      const int real = feats[f].real;
      // serial.rs:1538-1554: the by-node sample gates only the fold, not the splittable flags
      const uint8_t nm = p.bynode ? __ldcg(&J.used[(size_t)(1 + side) * p.F + f]) : (uint8_t)1;
      if (!searched || leaf < 0 || !u) continue;
      if (record && !stopped) J.splittable[(size_t)slot * p.F + f] = cs;
      if (nm) pick(a, make_pick(f, g, real, th));
    }
  }
  // the fold never adopts a NaN gain, so its order is total
  if (searched) a = warp_argmax(a, a.i >= 0, lane);
  if (lane == 0) ds.f[warp] = a;
  __syncthreads();
  if (warp != 0) return;
  if (stopped) {
    if (lane == 0) out->stop = 1;
    return;
  }
  // lanes 0 / 1: the new best of the smaller / larger leaf
  Pick nb = none;
  const int32_t my_leaf = lane == 0 ? leaf0 : leaf1;
  if (searched && lane < 2 && my_leaf >= 0) {
    Pick fa = none;
    for (int w = lane * (kDecideWarps / 2); w < (lane + 1) * (kDecideWarps / 2); ++w) pick(fa, ds.f[w]);
    // the fold starts from SplitInfo::default (gain -inf, feature -1) and replaces it only with a
    // better candidate
    const bool take = fa.i >= 0 && better_k(fa.k, fa.nan, fa.f, dkey(-CUDART_INF), false, -1);
    if (take)
      nb = Pick{my_leaf, fa.f, fa.k, fa.nan, fa.g, (long long)fa.i * 4294967296LL + (long long)(uint32_t)fa.pay};
    else
      nb = make_pick(my_leaf, -CUDART_INF, -1, (long long)-1 * 4294967296LL);
    if (record) {
      J.bgain[my_leaf] = nb.g;
      J.bfeat[my_leaf] = nb.f;
      J.bsplit[my_leaf] = nb.pay;
    }
  }
  // the leaf arg-max over the 8 warp partials (lanes 0..7) and the searched leaves (lanes 8, 9)
  const Pick moved = shfl_pick(nb, lane & 1, false);
  Pick w = lane < kDecideWarps ? ds.l[lane] : ((lane == 8 || lane == 9) ? moved : none);
  if (__any_sync(FULL, w.i >= 0 && w.nan)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) leaf_pick(w, shfl_pick(w, o, true));
  } else {
    w = warp_argmax(w, w.i >= 0, lane);
  }
  const int32_t inner = w.i >= 0 ? (int32_t)(w.pay >> 32) : -1;
  // serial.rs:611 — a best gain <= 0 stops the tree
  if ((!w.nan && w.k <= 0) || inner < 0) {
    if (lane == 0) {
      out->stop = 1;
      if (record) st->stop = 1;
    }
    return;
  }
  if (lane == 0) {
    const bool near = w.i < kDecideThreads;
    Decision d;
    d.stop = 0;
    d.leaf = w.i;
    d.inner = inner;
    d.thr = (uint32_t)(w.pay & 0xffffffffLL);
    d.begin = near ? ds.lb[w.i] : __ldcg(&J.leaf_begin[w.i]);
    d.count = near ? ds.lc[w.i] : __ldcg(&J.leaf_count[w.i]);
    d.buf = near ? ds.lbuf[w.i] : __ldcg(&J.leaf_buf[w.i]);
    d.depth = near ? ds.ld[w.i] : __ldcg(&J.leaf_depth[w.i]);
    d.pslot = near ? ds.lslot[w.i] : __ldcg(&J.leaf_slot[w.i]);
    d.sslot = ds.next_free;
    d.new_leaf = ds.tree_leaves;
    *out = d;
    if (record) {
      st->split_begin = d.begin;
      st->split_count = d.count;
      st->split_buf = d.buf;
      st->split_depth = d.depth;
      st->split_sslot = d.sslot;
      st->split_pslot = d.pslot;
      st->split_leaf = d.leaf;
      st->split_inner = d.inner;
      st->split_thr = d.thr;
      st->new_leaf = d.new_leaf;
    }
  }
}

// The whole decision on one CTA of kDecideThreads threads (the stable path's last search CTA).
__device__ void decide_split(const Job& J, const Params& p, const DevFeature* feats, bool record, Decision* out) {
  __shared__ DecideSmem ds;
  decide_leaves(J, p, ds);
  __syncthreads();
  decide_finish(J, p, feats, record, out, ds);
}

}  // namespace

}  // namespace bk

// Device grow-loop bookkeeping shared by the search and partition translation units:
// SerialTreeLearner::split after the partition (serial.rs:1685-1876) and BeforeFindBestSplit for
// the next iteration (serial.rs:779-825), including the histogram-pool slot choice
// (serial.rs:80-162 with a full pool: the larger child keeps the parent's slot).
#pragma once
#include <math_constants.h>

#include "bk_common.cuh"
#include "bk_math.cuh"

namespace bk {

__device__ __forceinline__ void before_find_best_split(const Job& J, const Params& p, JobState* st, int32_t left, int32_t right,
                                       int lane) {
  bool go = true;
  if (p.max_depth > 0 && J.leaf_depth[left] >= p.max_depth) go = false;
  int32_t nl = (int32_t)J.leaf_count[left];
  int32_t nr = right >= 0 ? (int32_t)J.leaf_count[right] : 0;
  if (go && nr < p.min_data * 2 && nl < p.min_data * 2) go = false;
  if (!go) {
    if (lane == 0) {
      J.bgain[left] = -CUDART_INF;
      if (right >= 0) J.bgain[right] = -CUDART_INF;
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
    st->hist_begin = J.leaf_begin[sl];
    st->hist_count = rows;
    st->hist_buf = J.leaf_buf[sl];
    if (rows == p.n) st->hist_rows_direct += rows;
    else st->hist_rows_gather += rows;
    st->hist_builds += 1;
  }
  // serial.rs:840-854 — features outside the tree's column sample are not searched; features the
  // parent could not split are skipped for both children.
  for (int f = lane; f < p.F; f += 32) {
    uint8_t u = parent_slot < 0 ? 1 : J.splittable[(size_t)parent_slot * p.F + f];
    J.used[f] = u & J.tree_mask[f];
    if (!u) J.splittable[(size_t)smaller_slot * p.F + f] = 0;
  }
  if (lane == 0) st->do_search = 1;
}

// What a split does to the leaf records once its left row count L is known
// (SerialTreeLearner::split, serial.rs:1685-1876, then BeforeFindBestSplit(left, right) of the
// next iteration, serial.rs:779-825): every value comes from the job state the decision wrote
// (split leaf, its row range, depth, the next free pool slot) and L, so any CTA can derive the
// children's row ranges without waiting for the bookkeeping below.
struct SplitOutcome {
  int32_t bl, nl, tl;   // the split leaf (keeps the left child), the new right leaf, leaves before the split
  int32_t sslot;        // the pool slot of the smaller child (the larger keeps the parent's)
  int32_t depth;        // depth of both children
  int32_t nbuf;         // index buffer of both children
  int64_t b, L, R;      // the parent's range start, the children's row counts
  bool go, left_smaller;
  __device__ int64_t hist_begin() const { return left_smaller ? b : b + L; }
  __device__ int64_t hist_count() const { return left_smaller ? L : R; }
};

__device__ __forceinline__ SplitOutcome split_outcome(const Params& p, const JobState* st, int64_t L) {
  SplitOutcome o;
  o.bl = st->split_leaf;
  o.nl = st->new_leaf;
  o.tl = st->new_leaf;  // the decision records the leaf count as the new leaf's index
  o.sslot = st->split_sslot;
  o.depth = st->split_depth + 1;
  o.nbuf = 1 - st->split_buf;
  o.b = st->split_begin;
  o.L = L;
  o.R = st->split_count - L;
  o.go = !(p.max_depth > 0 && o.depth >= p.max_depth);
  if (o.go && (int32_t)o.R < p.min_data * 2 && (int32_t)o.L < p.min_data * 2) o.go = false;
  o.left_smaller = (int32_t)o.L < (int32_t)o.R;
  return o;
}

// The children's sums and outputs from the split's candidate record: what the bookkeeping writes
// into leaf_sum (the smaller child first).
__device__ __forceinline__ void split_children(const Cand& info, const SplitOutcome& o, LeafSum* smaller,
                                               LeafSum* larger) {
  const LeafSum left{info.lsg, info.lsh, info.left_output, info.lint, (int32_t)o.L, 0};
  const LeafSum right{info.rsg, info.rsh, info.right_output, info.rint, (int32_t)o.R, 0};
  *smaller = o.left_smaller ? left : right;
  *larger = o.left_smaller ? right : left;
}

// One warp: the bookkeeping of a split (records, leaf arrays, pool slots, the next smaller /
// larger leaf and its row range, the skipped features). Every value is loaded first (independent
// loads in flight together), then every store is issued. It writes no job-state field that a
// split_outcome() reads, so CTAs of the same launch can still derive the outcome.
__device__ __forceinline__ void post_split_writes(const Job& J, const Params& p, const SplitOutcome& o, int lane) {
  JobState* st = J.st;
  // ---- loads ----
  const int64_t hdir = st->hist_rows_direct, hgat = st->hist_rows_gather, hbld = st->hist_builds;
  const int32_t pslot = J.leaf_slot[o.bl];
  Cand info = J.cand[(size_t)o.bl * p.F + st->split_inner];  // the chosen leaf's best split
  const int32_t miss = info.missing;
  info.left_count = (int32_t)o.L;
  info.right_count = (int32_t)o.R;
  const int32_t bl = o.bl, nl = o.nl;
  // serial.rs:1719-1722 — with interaction constraints, both children's paths gain the feature
  if (p.n_icons > 0) {
    uint32_t* pb = leaf_path_bits(J, p, bl);
    uint32_t* pn = leaf_path_bits(J, p, nl);
    const int32_t inner = info.inner;
    for (int w = lane; w < p.path_words; w += 32) {
      const uint32_t v = pb[w] | (w == (inner >> 5) ? (1u << (inner & 31)) : 0u);
      pn[w] = v;
      pb[w] = v;
    }
  }
  // lanes 0-7: word `lane` of a categorical split's left-bin bitset (serial.rs:1724-1759)
  if (lane < 8)
    J.records[o.tl - 1].cat_bins[lane] =
        info.categorical ? __ldcg(cand_cat_bits(J, p, o.bl, info.inner) + lane) : 0u;
  if (lane == 0) {
    J.leaf_count[bl] = o.L;
    J.leaf_begin[nl] = o.b + o.L;
    J.leaf_count[nl] = o.R;
    J.leaf_buf[bl] = o.nbuf;
    J.leaf_buf[nl] = o.nbuf;
    bk_split& r = J.records[o.tl - 1];
    r.leaf = bl;
    r.right_leaf = nl;
    r.inner_feature = info.inner;
    r.real_feature = info.feature;
    r.threshold = info.threshold;
    r.default_left = info.default_left;
    r.missing_type = miss;
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
    r.categorical = info.categorical;
    r._pad = 0;
    J.leaf_value[bl] = isnan(info.left_output) ? 0.0 : info.left_output;
    J.leaf_value[nl] = isnan(info.right_output) ? 0.0 : info.right_output;
    J.leaf_depth[nl] = o.depth;
    J.leaf_depth[bl] = o.depth;
    J.leaf_sum[bl] = LeafSum{info.lsg, info.lsh, info.left_output, info.lint, info.left_count, 0};
    J.leaf_sum[nl] = LeafSum{info.rsg, info.rsh, info.right_output, info.rint, info.right_count, 0};
    // the children's bests come from their search; without one both leaves drop out
    J.bgain[bl] = -CUDART_INF;
    J.bfeat[bl] = info.feature;
    st->tree_leaves = o.tl + 1;
    if (!o.go) {
      J.bgain[nl] = -CUDART_INF;
      st->do_search = 0;
    } else {
      st->next_free = o.sslot + 1;
      J.leaf_slot[o.left_smaller ? nl : bl] = pslot;
      J.leaf_slot[o.left_smaller ? bl : nl] = o.sslot;
      st->smaller_leaf = o.left_smaller ? bl : nl;
      st->larger_leaf = o.left_smaller ? nl : bl;
      st->smaller_slot = o.sslot;
      st->larger_slot = pslot;
      st->parent_slot = pslot;
      st->use_subtract = 1;
      const int64_t rows = o.hist_count();
      st->hist_begin = o.hist_begin();
      st->hist_count = rows;
      st->hist_buf = o.nbuf;
      if (rows == p.n) st->hist_rows_direct = hdir + rows;
      else st->hist_rows_gather = hgat + rows;
      st->hist_builds = hbld + 1;
      st->do_search = 1;
    }
  }
  if (o.go) {
    // serial.rs:840-854 — features outside the tree's column sample are not searched; features
    // the parent could not split are skipped for both children
    for (int f = lane; f < p.F; f += 32) {
      uint8_t u = J.splittable[(size_t)pslot * p.F + f];
      J.used[f] = u & J.tree_mask[f];
      if (!u) J.splittable[(size_t)o.sslot * p.F + f] = 0;
    }
  }
}

// Runs on the first warp of the last CTA of the stable partition: the split's bookkeeping with L
// from the partition's count.
__device__ __forceinline__ void post_split_body(const Job& J, const Params& p, const DevFeature* feats) {
  (void)feats;
  const SplitOutcome o = split_outcome(p, J.st, __ldcg(&J.st->total_left));
  post_split_writes(J, p, o, (int)threadIdx.x);
}

}  // namespace bk

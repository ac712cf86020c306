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
  // serial.rs:840-854 — features the parent could not split are skipped for both children.
  for (int f = lane; f < p.F; f += 32) {
    uint8_t u = parent_slot < 0 ? 1 : J.splittable[(size_t)parent_slot * p.F + f];
    J.used[f] = u;
    if (!u) J.splittable[(size_t)smaller_slot * p.F + f] = 0;
  }
  if (lane == 0) st->do_search = 1;
}

// Runs on the first warp of the last CTA of the partition scatter: SerialTreeLearner::split's
// bookkeeping after DataPartition::split, then BeforeFindBestSplit(left, right) of the next
// iteration. Every value is loaded first (independent loads in flight together), then every
// store is issued, so the serial tail of a split costs about one memory round trip.
__device__ __forceinline__ void post_split_body(const Job& J, const Params& p, const DevFeature* feats) {
  JobState* st = J.st;
  const int lane = threadIdx.x;
  // ---- loads ----
  const int32_t bl = st->split_leaf, nl = st->new_leaf, tl = st->tree_leaves, nf = st->next_free;
  const int64_t L = __ldcg(&st->total_left);  // written by another CTA of the scatter
  const int64_t hdir = st->hist_rows_direct, hgat = st->hist_rows_gather, hbld = st->hist_builds;
  const int64_t b = st->split_begin, c = st->split_count;
  const int32_t buf = st->split_buf, depth = J.leaf_depth[bl], pslot = J.leaf_slot[bl];
  Cand info = J.cand[(size_t)bl * p.F + st->split_inner];  // the chosen leaf's best split
  const int32_t miss = info.missing;
  // ---- the split (serial.rs:1685-1876) ----
  const int64_t R = c - L;
  info.left_count = (int32_t)L;
  info.right_count = (int32_t)R;
  const int32_t nd = depth + 1;  // tree.leaf_depth of both children
  // ---- BeforeFindBestSplit(bl, nl) (serial.rs:779-825) ----
  bool go = !(p.max_depth > 0 && nd >= p.max_depth);
  const int32_t nleft = (int32_t)L, nright = (int32_t)R;
  if (go && nright < p.min_data * 2 && nleft < p.min_data * 2) go = false;
  const bool left_smaller = nleft < nright;
  const int32_t sslot = nf;  // the smaller child gets a new slot; the larger keeps the parent's
  if (lane == 0) {
    J.leaf_count[bl] = L;
    J.leaf_begin[nl] = b + L;
    J.leaf_count[nl] = R;
    J.leaf_buf[bl] = 1 - buf;
    J.leaf_buf[nl] = 1 - buf;
    bk_split& r = J.records[tl - 1];
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
    J.leaf_value[bl] = isnan(info.left_output) ? 0.0 : info.left_output;
    J.leaf_value[nl] = isnan(info.right_output) ? 0.0 : info.right_output;
    J.leaf_depth[nl] = nd;
    J.leaf_depth[bl] = nd;
    J.leaf_sum[bl] = LeafSum{info.lsg, info.lsh, info.left_output, info.lint, info.left_count, 0};
    J.leaf_sum[nl] = LeafSum{info.rsg, info.rsh, info.right_output, info.rint, info.right_count, 0};
    // the children's bests come from their search; without one both leaves drop out
    J.bgain[bl] = -CUDART_INF;
    J.bfeat[bl] = info.feature;
    st->tree_leaves = tl + 1;
    if (!go) {
      J.bgain[nl] = -CUDART_INF;
      st->do_search = 0;
    } else {
      st->next_free = nf + 1;
      J.leaf_slot[left_smaller ? nl : bl] = pslot;
      J.leaf_slot[left_smaller ? bl : nl] = sslot;
      st->smaller_leaf = left_smaller ? bl : nl;
      st->larger_leaf = left_smaller ? nl : bl;
      st->smaller_slot = sslot;
      st->larger_slot = pslot;
      st->parent_slot = pslot;
      st->use_subtract = 1;
      const int64_t rows = left_smaller ? L : R;
      st->hist_begin = left_smaller ? b : b + L;
      st->hist_count = rows;
      st->hist_buf = 1 - buf;
      if (rows == p.n) st->hist_rows_direct = hdir + rows;
      else st->hist_rows_gather = hgat + rows;
      st->hist_builds = hbld + 1;
      st->do_search = 1;
    }
  }
  if (go) {
    // serial.rs:840-854 — features the parent could not split are skipped for both children
    for (int f = lane; f < p.F; f += 32) {
      uint8_t u = J.splittable[(size_t)pslot * p.F + f];
      J.used[f] = u;
      if (!u) J.splittable[(size_t)sslot * p.F + f] = 0;
    }
  }
}

}  // namespace bk

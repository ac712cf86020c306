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
      J.best[left].gain = -CUDART_INF;
      J.bgain[left] = -CUDART_INF;
      if (right >= 0) {
        J.best[right].gain = -CUDART_INF;
        J.bgain[right] = -CUDART_INF;
      }
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

// Runs on the first warp of the last CTA of the partition scatter.
__device__ __forceinline__ void post_split_body(const Job& J, const Params& p, const DevFeature* feats) {
  JobState* st = J.st;
  const int lane = threadIdx.x;
  const int32_t bl = st->split_leaf, nl = st->new_leaf;
  const int64_t L = __ldcg(&st->total_left);  // written by another CTA of the scatter
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
    J.bgain[bl] = info.gain;
    J.bfeat[bl] = info.feature;
    st->tree_leaves += 1;
  }
  __syncwarp();
  before_find_best_split(J, p, st, bl, nl, lane);
}


}  // namespace bk

// Prediction of binned rows through a trained tree on the device: the replay that
// SerialTreeLearner::add_prediction_for_rows performs for rows outside the training partition
// (serial.rs:2009-2041), with each split's routing rule (data_partition.rs:299-410) evaluated on
// the rows' stored bins. Rows binned with the training bin mappers land in the same leaves as
// the reference's threshold comparisons on raw values (a value is <= the bin's upper bound
// exactly when its bin is <= the threshold bin). A categorical split routes by the bitset of its
// left bins over the feature's bin mapper (data_partition.rs:264-300, route_bin :367-377): stored
// bin 0 holds the most frequent bin's rows and goes left when that bin is not 0 and is in the
// set; stored bin b looks up bit b - 1 + offset.
#include <cuda_runtime.h>

#include "bk_math.cuh"

namespace bk {

namespace {

__global__ void k_predict_tree(const DevFeature* __restrict__ feats, int32_t num_leaves,
                               const int32_t* __restrict__ tree, const double* __restrict__ leaf_value,
                               const uint8_t* __restrict__ bins, int64_t m, double* __restrict__ score) {
  // tree: [left_child | right_child | split_feature_inner | threshold_in_bin | decision_type],
  // then 8 words of left-bin bitset per node (categorical splits, decision_type bit 0)
  const int32_t ni = num_leaves - 1;
  const int32_t* lc = tree;
  const int32_t* rc = tree + ni;
  const int32_t* sf = tree + 2 * ni;
  const int32_t* th = tree + 3 * ni;
  const int32_t* dt = tree + 4 * ni;
  const uint32_t* cb = reinterpret_cast<const uint32_t*>(tree + 5 * ni);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t node = num_leaves > 1 ? 0 : -1;
    int guard = 0;
    while (node >= 0 && guard++ < num_leaves) {
      const int32_t f = sf[node];
      const uint32_t bin = bins[(size_t)f * (size_t)m + i];
      const DevFeature& fm = feats[f];
      bool left;
      if (dt[node] & 1) {
        const uint32_t pos = bin == 0 ? (uint32_t)fm.mfb : bin - 1 + (uint32_t)fm.offset;
        const bool set = pos < 256u && ((cb[(size_t)node * 8 + (pos >> 5)] >> (pos & 31)) & 1u) != 0u;
        left = (int)bin < fm.gbins && set && (bin != 0 || fm.mfb > 0);
      } else {
        left = route_bin(fm, (uint32_t)th[node], (dt[node] & 2) != 0, bin) != 0;
      }
      node = left ? lc[node] : rc[node];
    }
    score[i] += leaf_value[node < 0 ? ~node : 0];
  }
}

}  // namespace

cudaError_t predict_tree(const DevFeature* feats, int32_t num_leaves, const int32_t* d_tree, const double* d_leaf_value,
                         const uint8_t* bins, int64_t m, double* score, cudaStream_t s) {
  k_predict_tree<<<1024, 256, 0, s>>>(feats, num_leaves, d_tree, d_leaf_value, bins, m, score);
  return cudaGetLastError();
}

}  // namespace bk

// Shared device-side definitions of the GB300 tree learner.
//
// Layout in HBM (one learner, `n` rows, `F` inner features, `T = ceil(F / 32)` feature tiles,
// `B` = the largest stored-bin count of any feature, rounded up to a multiple of 8):
//   bins_rt   uint8 [n][S]       (S = Σ w_t rounded up to a multiple of 64: rows on 64-byte bursts)
//                                row-tiled stored bins: one w_t-byte run per (row, tile) — 32 bytes
//                                for a tile of 8-bit bins, 16 for a tile of 4-bit bins (every
//                                feature of the tile has at most 16 group bins) — so a gathered
//                                row of a sparse leaf is one sector read per tile, and the T
//                                histogram CTAs of a row chunk, which run side by side, read
//                                neighbouring sectors of the same lines;
//   bins_tm   [T] x uint8 [n][w_t]   the same runs tile-major: the root and dense leaves (a
//                                quarter of the rows or more) stream each tile contiguously;
//   bins_cm   uint8 [F][n]       column-major stored bins, read by the partition (one byte/row);
//   pool      [L][T][B][32]      histogram pool, one slot per leaf (serial.rs:80-162 with a full
//                                pool): double2 (grad, hess) on the float path, int64
//                                (grad << 32) + hess on the quantized path;
// and per job (one tree of the K trees grown together): gradients, packed int8 gradients,
// two row-index buffers (ping-pong between a leaf and its children) and, on the quantized path,
// the packed values in the same leaf order beside them (the partition moves them with the row
// indices, so a histogram reads them contiguously instead of gathering one per row), leaf
// bookkeeping.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bkgpu.h"

// Sets the calling thread's message for bk_last_error() (defined in bk_learner.cu).
void bk_set_last_error(const char* msg);

namespace bk {

constexpr int TILE = 32;
// meta.rs:7 — kEpsilon = 1e-15f widened to double; meta.rs:4 — kZeroThreshold = 1e-35f.
#define BK_EPS ((double)1e-15f)
#define BK_ZERO_THRESHOLD ((double)1e-35f)

struct DevFeature {
  int32_t num_bin, missing, default_bin, mfb;
  int32_t offset;  // 1 when the most frequent bin is 0 (its bin is not in the histogram slice)
  int32_t gbins;   // stored bins of the feature's group: 1 + num_bin - offset
  int32_t real;    // real (original) column index
  int32_t len;     // searched slice length: num_bin - offset
  double penalty;
  int32_t cat;     // 1: categorical (BinType::Categorical)
  int32_t _pad;
};

// A split candidate of one (leaf, feature): SplitInfo (split_info.rs:9-31) plus its
// splittable flag and the inner feature index.
struct Cand {
  double gain, left_output, right_output, lsg, lsh, rsg, rsh;
  int64_t lint, rint;
  int32_t feature, inner;
  uint32_t threshold;
  int32_t left_count, right_count, default_left, splittable, missing;  // missing: the feature's missing type
  int32_t categorical;  // 1: a categorical split, its left bins in cand_cat_bits()
};

// The stored-bin layout of one 32-feature tile in the two row-tiled copies (static per learner):
// a tile whose features all have at most 16 group bins holds 4-bit bins (16 bytes per row: byte k
// = feature 2k in the low nibble, feature 2k + 1 in the high one, as io/bin_data.rs:20-30 stores
// groups of <= 16 bins two to a byte); any other tile one byte per bin, 32 bytes per row, or 16
// when it holds at most 16 features (the last tile of a feature count that is not a multiple of 32).
struct TileGeom {
  int32_t bins;    // group bins the tile's shared histogram holds: its largest feature's, rounded up to 8
  int32_t nibble;  // 1: 4-bit stored bins
  int32_t width;   // bytes per row: 16 or 32
  int32_t _pad;
  int64_t rt_off;  // byte offset of the tile in a row of bins_rt
  int64_t tm_off;  // byte offset of the tile's [n][width] block in bins_tm
};

__host__ __device__ __forceinline__ int tile_width(const TileGeom& g) { return g.width; }

// LeafSplits (serial.rs:53-76).
struct LeafSum {
  double sg, sh, weight;
  int64_t int_sum;
  int32_t num_data, _pad;
};

struct Params {
  double l1, l2, max_delta, smooth, min_hess, min_gain;
  int32_t min_data, fused, use_l1, use_max, use_smooth, quant;
  int32_t const_hess, num_leaves, max_depth, F;
  int32_t T, B, quant_bins, stochastic;
  int32_t renew, part_grid, pdl;  // pdl: launch the grow-loop kernels with programmatic dependence
  int32_t hist_min_rows;          // fewest rows a histogram CTA takes (launch shape, autotuned)
  int32_t rt_stride;              // bytes per row of bins_rt: the widths of all tiles
  int32_t search_narrow;          // 1: every feature is numerical with at most 63 searched bins (the
                                  //    plain single-pass search runs in 64-thread CTAs)
  const TileGeom* tiles;          // [T] the tiles' layouts
  int64_t n;
  // CatParams of the categorical search (feature_histogram.rs:1146-1163)
  double cat_smooth, cat_l2;
  int32_t max_cat_threshold, max_cat_to_onehot, min_data_per_group;
  int32_t bynode;  // 1: every searched leaf gets a by-node feature mask (Job::used[F..3F)): a sample
                   //    and / or its interaction constraints
  int32_t n_icons;     // interaction constraints: how many feature sets, of `path_words` words each
  int32_t path_words;  // words of a feature bitset: ceil(F / 32)
  const uint32_t* icons;  // [n_icons][path_words] inner-feature bitsets
};

// Per-leaf constants of one searched leaf (FindBestThreshold's preamble, feature_histogram.rs:
// 219-240 / 673-700): computed once per search, before it, by one CTA of the histogram launch.
struct LeafConst {
  double sum_g, sum_h, parent, mgs, cnt_factor;  // mgs = min_gain_shift
  int64_t first_x, brk_x;  // quantized path: validity thresholds on the accumulated hessian
  float mgs_up, mgs_dn;    // min_gain_shift rounded up / down to fp32
  float gsf, hsf, l2f;     // fp32 copies of the gradient / hessian scales and lambda_l2
  float _pad;
  double gs, hs;           // quantized path: the gradient / hessian scales
  LeafSum ls;              // the leaf's sums (its LeafSplits), as leaf_sum[leaf] holds them
};

// Per-job control block, written and read only by kernels (the device-resident grow loop).
struct JobState {
  int32_t stop, do_search, tree_leaves, disc_ok;
  int32_t smaller_leaf, larger_leaf, smaller_slot, larger_slot;
  int32_t parent_slot, use_subtract, next_free, split_leaf;
  int32_t split_inner, new_leaf, use_rows;
  uint32_t split_thr;  // threshold of the chosen split | default_left << 31
  int64_t root_count, total_left;
  int64_t pcnt[2][2];  // single-pass partition: rows placed from the front / back, per split parity
  int64_t hist_begin, hist_count;  // the smaller leaf's row range and index buffer, for the histogram
  int32_t hist_buf, split_buf;
  int64_t split_begin, split_count;  // the chosen leaf's row range and index buffer, for the partition
  int32_t split_depth, split_sslot;  // the chosen leaf's depth and the pool slot its smaller child gets
  double gscale, hscale, inv_g, inv_h;
  double root_output;
  uint32_t start_pos, red_maxg, red_maxh, red_flags;
  int32_t mt_idx;
  int32_t split_pslot;  // the chosen leaf's pool slot, which its larger child keeps
  int64_t hist_rows_direct, hist_rows_gather, hist_builds;  // work done by the histogram kernels
  uint32_t search_done, part_done;  // CTAs finished in the current search / scatter launch
  // by-node column sample (col_sampler.rs:109-177): the sampler's LCG state, whether a by-tree
  // sample is active, the by-node fraction
  uint32_t col_rng;
  int32_t bytree_on;
  double bynode_fraction;
  uint32_t mt[624];
};

// Device pointers of one job.
struct Job {
  JobState* st;
  const float* g;
  const float* h;
  int16_t* packed;
  int32_t* idx0;
  int32_t* idx1;
  int16_t* pk0;  // quantized path: packed values in the leaf order of idx0 / idx1 (not the root's)
  int16_t* pk1;
  int64_t* leaf_begin;
  int64_t* leaf_count;
  int32_t* leaf_buf;
  int32_t* leaf_depth;
  int32_t* leaf_slot;
  LeafSum* leaf_sum;
  double* bgain;       // [L]   gain of each leaf's best split (the arg-max reads these)
  int32_t* bfeat;      // [L]   real feature of each leaf's best split
  Cand* cand;          // [L][F] the candidate of every searched (leaf, feature); a leaf's best split is
                       //        cand[leaf][inner feature of bsplit[leaf]]
  double* cgain;       // [2][F] gains of the current search's candidates (compact copy for the fold)
  uint8_t* csplit;     // [2][F] splittable flags of the current search's candidates
  uint32_t* cthr;      // [2][F] threshold | default_left << 31 of cand[]
  int64_t* bsplit;     // [L]   inner feature << 32 | threshold | default_left << 31 of each leaf's best split
  LeafConst* lconst;   // [2]   constants of the smaller / larger leaf of the current search
  uint8_t* splittable; // [L][F]
  uint8_t* used;       // [4][F] features searched in the current step; the by-node masks of the
                       //        smaller / larger leaf; the sample's scratch; then [L][path_words]
                       //        uint32 bitsets of the features on the path to each leaf
  uint8_t* tree_mask;  // [F]   features the tree may split on (by-tree column sample), 1 by default
  bk_split* records;   // [L-1]
  double* leaf_value;  // [L]
  void* pool;          // [L][T][B][32]
  int64_t* part_cnt;   // [part_grid] partition block counts (scratch)
  double* red;         // reduction partials (scratch)
  int64_t* ired;       // integer reduction partials (scratch)
};

// The jobs of one grow-loop launch, passed by value: the kernel parameters sit in the constant
// bank, so a kernel reaches its job's buffers without a global-memory round trip after it starts.
// Sixteen jobs (about 4 KB of parameters) cover every class tree of a multiclass iteration of up
// to 16 classes in one launch per kernel; a learner with more jobs launches each grow-loop kernel
// once per group of sixteen.
constexpr int kJobsPerLaunch = 16;
struct JobTable {
  Job job[kJobsPerLaunch];
};
static_assert(sizeof(JobTable) <= 4096, "the job table of a grow-loop launch stays within 4 KB of parameters");

// Calls f(table, jobs in it) for each group of up to kJobsPerLaunch consecutive host-side jobs.
template <typename F>
inline void for_job_groups(const Job* h_jobs, int num_jobs, F f) {
  for (int z0 = 0; z0 < num_jobs; z0 += kJobsPerLaunch) {
    JobTable t = {};
    const int nz = num_jobs - z0 < kJobsPerLaunch ? num_jobs - z0 : kJobsPerLaunch;
    for (int i = 0; i < nz; ++i) t.job[i] = h_jobs[z0 + i];
    f(t, nz);
  }
}

// The bin bitsets of categorical candidates, stored after the [L][F] candidates in the same
// allocation (8 words per (leaf, feature); written only by categorical searches).
__host__ __device__ __forceinline__ size_t cand_cat_words(int num_leaves, int F) {
  return (size_t)num_leaves * (size_t)F * 8;
}
__device__ __forceinline__ uint32_t* cand_cat_bits(const Job& J, const Params& p, int32_t leaf, int32_t f) {
  return reinterpret_cast<uint32_t*>(J.cand + (size_t)p.num_leaves * p.F) + ((size_t)leaf * p.F + f) * 8;
}

// The features on the path to `leaf` (SerialTreeLearner::branch_features, serial.rs:233-234) as a
// bitset over inner features, kept only with interaction constraints.
__device__ __forceinline__ uint32_t* leaf_path_bits(const Job& J, const Params& p, int32_t leaf) {
  return reinterpret_cast<uint32_t*>(J.used + 4 * (size_t)p.F) + (size_t)leaf * p.path_words;
}

__device__ __forceinline__ const int32_t* leaf_idx(const Job& J, int32_t buf) { return buf ? J.idx1 : J.idx0; }
__device__ __forceinline__ int32_t* leaf_idx_w(const Job& J, int32_t buf) { return buf ? J.idx1 : J.idx0; }
__device__ __forceinline__ int16_t* leaf_pk(const Job& J, int32_t buf) { return buf ? J.pk1 : J.pk0; }

__host__ __device__ __forceinline__ int64_t ceil_div64(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---- launchers (defined in the kernel translation units) ----
constexpr int kMaxPartGrid = 1024;  // most partition CTAs per launch (the per-CTA count scratch)

struct HistLaunch {
  int blocks_per_tile;
  int threads;
  size_t smem;
  int flush_rounds;  // quantized: rounds of 32*warps rows between 16-bit -> 32-bit flushes (0: wide)
  int direct_rows;   // quantized: a CTA with at most this many rows adds each (row, feature) to the
                     // pool slot with a global atomic instead of through a shared histogram
  int cluster = 1;   // quantized: CTAs of a tile per thread-block cluster, which add up their shared
                     // histograms through distributed shared memory before one flush (1: none)
};
// BinsCheck over device columns: the smallest flat index (feature * n + row) of a stored bin
// outside its feature's range, or INT64_MAX (bk_binning.cu). Synchronizes `s`.
cudaError_t check_bins_device(const uint8_t* bins, int64_t n, int32_t F, const DevFeature* d_feat,
                              int64_t* first_bad, cudaStream_t s);
// post: the previous split came from the single-pass partition, whose counter pair `par` holds
// its left total; the launch applies that split's bookkeeping.
void launch_hist(const Job* h_jobs, int num_jobs, const Params& p, const uint8_t* bins_rt, const uint8_t* bins_tm,
                 const HistLaunch& hl, int post, int par, cudaStream_t s);
size_t hist_smem_bytes(const Params& p, int threads, bool quant, bool wide);

// The bookkeeping of the last split of a tree partitioned in one pass (counter pair `par`).
void launch_apply_split(const Job* h_jobs, int num_jobs, const Params& p, int par, cudaStream_t s);
// clear_par >= 0: the launch zeroes that single-pass partition counter pair first. decide: its
// last CTA decides and records the split (else the single-pass partition decides it).
void launch_search(const Job* h_jobs, int num_jobs, const Params& p, const DevFeature* feats, int clear_par,
                   bool decide, int post, cudaStream_t s);
// stable: the two-kernel compaction whose last CTA applies the split's bookkeeping; otherwise the
// single-pass partition, counting into the counter pair `par` (the split index's parity), whose
// bookkeeping the next histogram launch applies.
// decide (single-pass only): every CTA decides the split from the search's records first.
void launch_partition(const Job* h_jobs, int num_jobs, const Params& p, const uint8_t* bins_cm,
                      const DevFeature* feats, bool stable, int par, bool decide, cudaStream_t s);

cudaError_t hist_set_smem_attrs(size_t smem);

// bk_prep.cu
void launch_init_rows(const Job* d_jobs, int num_jobs, const Params& p, const int32_t* rows, cudaStream_t s);
void launch_discretize(const Job* d_jobs, int num_jobs, const Params& p, const double* noise_g, const double* noise_h,
                       cudaStream_t s);
void launch_root_sums(const Job* d_jobs, int num_jobs, const Params& p, int exact_quant_root, cudaStream_t s);
void launch_renew(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s);
void launch_add_score(const Job* d_jobs, int num_jobs, const Params& p, const double* leaf_vals, double* score,
                      cudaStream_t s);
void launch_add_score_own(const Job* d_jobs, int num_jobs, const Params& p, double rate, double* score,
                          cudaStream_t s);
void launch_row_leaf(const Job* d_jobs, int num_jobs, const Params& p, int32_t* out, cudaStream_t s);
void launch_mt_seed(const Job* d_jobs, int num_jobs, uint32_t seed, cudaStream_t s);
constexpr int kRootGrid = 256;

// bk_predict.cu
cudaError_t predict_tree(const DevFeature* feats, int32_t num_leaves, const int32_t* d_tree, const double* d_leaf_value,
                         const uint8_t* bins, int64_t m, double* score, cudaStream_t s);

// bk_objective.cu
// Row weights (device f32 [n] or null: Metadata::weights) and the binary objective's label
// weights of the negative and positive class (BinaryLogloss::label_weights, binary.rs:33-52).
struct ObjectiveWeights {
  const float* row = nullptr;
  double label_neg = 1.0, label_pos = 1.0;
};
// bad_label: device counter of multiclass labels outside [0, K) (kind 2 only)
cudaError_t objective_gradients(int kind, const double* score, const float* label, int64_t n, int K, double sigmoid,
                                const ObjectiveWeights& ow, float* g, float* h, int32_t* bad_label, cudaStream_t s);
cudaError_t objective_loss(int kind, const double* score, const float* label, int64_t n, int K, double* partial,
                           int grid, int32_t* bad_label, cudaStream_t s);
void launch_tree_begin(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s);

}  // namespace bk

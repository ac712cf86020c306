/* bkgpu.h — C ABI of the GB300 tree learner for bankai-lightgbm's histogram hot path.
 *
 * The reference has no trait for its tree learner: `Trainer` calls the concrete method set of
 * `SerialTreeLearner` (crates/lgbm-core/src/treelearner/serial.rs:183-2044). Each entry point
 * below replaces one of those methods (cited per function) and takes plain pointers and sizes,
 * so a Rust `extern "C"` block can bind it directly.
 *
 * Conventions (mirroring the reference's c_api, crates/lgbm-capi/src/lib.rs:1-8,78):
 *   - every function returns 0 on success and -1 on failure; bk_last_error() then holds a
 *     message for the calling thread;
 *   - calls on one learner must not overlap (the reference runs one tree at a time per
 *     learner, serial.rs:569-576); all calls are synchronous unless stated;
 *   - "host" pointers are ordinary CPU memory; "device" pointers are CUDA global memory of the
 *     learner's device, selected by the `on_device` flags.
 */
#ifndef BKGPU_H
#define BKGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One inner (used) feature: the BinMapper facts the learner reads (io/bin.rs:21-36) plus the
 * real column index (io/dataset.rs:84-93 real_feature_idx) and its split penalty
 * (feature_contri). Stored bins follow io/dataset.rs:633-685: rows whose bin equals
 * most_freq_bin hold 0, other rows hold bin + 1 - (most_freq_bin == 0). */
typedef struct {
  int32_t num_bin;
  int32_t missing_type; /* 0 none, 1 zero, 2 NaN (meta.rs:10-16) */
  int32_t default_bin;
  int32_t most_freq_bin;
  double penalty;
  int32_t real_feature;
  int32_t bin_type; /* 0 numerical, 1 categorical (meta.rs BinType) */
} bk_feature;

/* The Config fields the tree learner reads (config/auto.rs). `num_threads` is the reference's
 * thread count, used only to seed stochastic-rounding noise per block exactly as the reference
 * does (gradient_discretizer/mod.rs:87-106). `fused_madd` selects the rounding of the
 * reference's `madd` (utils/common.rs:207-216): 1 = fused, as the aarch64 build; 0 = unfused.
 * The last five fields are the categorical search's CatParams (treelearner/feature_histogram.rs:
 * 1146-1163; defaults 4, 32, 10.0, 10.0, 100 in config/auto.rs:214-218). */
typedef struct {
  int32_t num_leaves, max_depth, min_data_in_leaf, _pad0;
  double min_sum_hessian_in_leaf, lambda_l1, lambda_l2, max_delta_step, path_smooth, min_gain_to_split;
  int32_t use_quantized_grad, num_grad_quant_bins, quant_train_renew_leaf, stochastic_rounding;
  int32_t seed, num_threads, fused_madd, is_constant_hessian;
  int32_t max_cat_to_onehot, max_cat_threshold;
  double cat_smooth, cat_l2;
  int32_t min_data_per_group, _pad1;
} bk_config;

/* One split: the arguments of Tree::split_numerical (tree.rs:361-403) or, for a categorical
 * feature, Tree::split_categorical (tree.rs:405-443), as computed by SerialTreeLearner::split
 * (serial.rs:1685-1876). Counts are the partition's actual counts. */
typedef struct {
  int32_t leaf, right_leaf, inner_feature, real_feature;
  uint32_t threshold; /* numerical: bin; the host maps it with BinMapper::bin_to_value */
  int32_t default_left, missing_type, left_count, right_count;
  double left_output, right_output, left_sum_gradient, left_sum_hessian, right_sum_gradient, right_sum_hessian;
  double gain; /* without min_gain_to_split; the tree stores (gain + min_gain_to_split) as f32 */
  int64_t left_int_sum, right_int_sum; /* quantized path: (grad << 32) | hess; 0 otherwise */
  int32_t categorical; /* 1: categorical split (serial.rs:1724-1759) */
  int32_t _pad;
  uint32_t cat_bins[8]; /* categorical: bitset of the bins that go left (bit b = bin b, construct_bitset of
                         * cat_threshold); the host maps the bins to categories with bin_to_value and builds
                         * the tree's category bitset */
} bk_split;

typedef struct bk_learner bk_learner;
typedef struct bk_learner_group bk_learner_group;

/* Replaces SerialTreeLearner::new (serial.rs:284-565). `bins` is column-major uint8
 * [num_features][num_data] of stored bins. `num_jobs` trees are grown per train call over the
 * same dataset (all K class trees of one multiclass iteration, objective/multiclass.rs). */
int bk_learner_create(const bk_feature* features, int32_t num_features, const uint8_t* bins, int64_t num_data,
                      const bk_config* config, int32_t num_jobs, bk_learner** out);

/* As bk_learner_create, with `bins` in device memory ([num_features][num_data] stored bins,
 * e.g. written by bk_bin_dense_device); the learner copies them and checks them on the device. */
int bk_learner_create_device_bins(const bk_feature* features, int32_t num_features, const uint8_t* bins,
                                  int64_t num_data, const bk_config* config, int32_t num_jobs, bk_learner** out);

/* Dense bin construction on the device: Dataset::from_dense's fill_dense (io/dataset.rs:633-685)
 * with BinMapper::value_to_bin (io/bin.rs:558-589) for every value, for bin mappers found on the
 * host (BinMapper::find_bin over a row sample, io/bin.rs:342-554; the held-out form is
 * from_dense_reference, io/dataset.rs:987-1003). values: device memory, row-major
 * [num_data][num_columns], value_type 0 = f64, 1 = f32. features: the used features' bin mappers
 * (real_feature = their column); upper_bounds: host, feature f's num_bin bounds at
 * upper_bounds[bound_offsets[f]], bound_offsets[num_features] in total. out: device
 * [num_features][num_data] stored bins (the most frequent bin stored as 0). Runs on `stream`
 * (a cudaStream_t, NULL for the default stream) and returns when the bins are written. */
int bk_bin_dense_device(const void* values, int32_t value_type, int64_t num_data, int32_t num_columns,
                        const bk_feature* features, int32_t num_features, const double* upper_bounds,
                        const int32_t* bound_offsets, uint8_t* out, void* stream);

/* Replaces SerialTreeLearner::train (serial.rs:569-628) for `num_jobs` trees at once.
 * gradients/hessians: [num_jobs][num_data] f32, host or device (on_device). rows: ascending
 * bagged row ids (num_rows of them) or NULL for all rows, host memory.
 * Outputs (host): splits [num_jobs][num_leaves-1], leaf_values [num_jobs][num_leaves] (the tree's
 * leaf outputs before shrinkage, after the quantized leaf renewal), root_outputs [num_jobs],
 * num_leaves_out [num_jobs]. */
int bk_learner_train(bk_learner* learner, const float* gradients, const float* hessians, int32_t on_device,
                     const int32_t* rows, int64_t num_rows, bk_split* splits, double* leaf_values,
                     double* root_outputs, int32_t* num_leaves_out);

/* Many independent boosting jobs at once: one bk_learner_train call (all rows, no bagging) for
 * each of `count` distinct learners — each with its own dataset, shape and config — queued on
 * the learners' own streams before any is waited for, so their grow loops run concurrently on
 * the device; then, if `scores` is not NULL, each learner's score update with its new trees
 * (train.rs:776-785: leaf outputs times `shrinkage`, values within kZeroThreshold of 0 set to 0
 * as Tree::apply_shrinkage does, tree.rs:446-463; a one-leaf tree adds nothing).
 * Per learner i: gradients[i] / hessians[i] as in bk_learner_train (host or device, on_device);
 * scores[i]: device f64 [num_jobs][num_data]; splits[i], leaf_values[i], root_outputs[i],
 * num_leaves_out[i]: host outputs as in bk_learner_train (each array of pointers may be NULL).
 * Replaces the per-job calls of SerialTreeLearner::train (serial.rs:569-628) and
 * add_prediction_to_score (serial.rs:1974-1990) that a host running many Boosters would make
 * one after another. Returns after every learner has finished. */
int bk_learners_train_batch(bk_learner* const* learners, int32_t count, const float* const* gradients,
                            const float* const* hessians, int32_t on_device, double shrinkage, double* const* scores,
                            bk_split* const* splits, double* const* leaf_values, double* const* root_outputs,
                            int32_t* const* num_leaves_out);

/* A fixed set of learners whose iterations run as one CUDA graph (GB300-only; the reference's
 * counterpart is the same as bk_learners_train_batch's: one SerialTreeLearner::train +
 * add_prediction_to_score per Booster, serial.rs:569-628, :1974-1990). Every learner's iteration
 * — the grow loop of its trees, the score update, the readback of its results — is one branch of
 * the graph, issued on the learner's own stream; one graph launch runs all of them with no host
 * work between their kernels. The learners keep their own datasets, shapes and configs; they must
 * share one device, appear once, use the graph form (loop mode 1) and have phase timing off when
 * trained. The graph is captured on the first bk_learner_group_train call and again whenever a
 * member's launch parameters change (launch shape, overlap, constraints, by-node sampling) or the
 * call's input pointers or shrinkage differ from the captured ones. A learner of a group may also
 * be used on its own, but never while a group call that holds it is running. */
int bk_learner_group_create(bk_learner* const* learners, int32_t count, bk_learner_group** out);

/* One iteration of every learner of the group, as bk_learners_train_batch does it with
 * on_device = 1: gradients[i] / hessians[i] device f32 [num_jobs][num_data] of learner i,
 * scores[i] device f64 [num_jobs][num_data] (the array may be NULL: no score update), outputs as in
 * bk_learners_train_batch. It runs after the work already queued on each member's stream (such as
 * bk_learner_objective_gradients). Synchronous. */
int bk_learner_group_train(bk_learner_group* group, const float* const* gradients, const float* const* hessians,
                           double shrinkage, double* const* scores, bk_split* const* splits,
                           double* const* leaf_values, double* const* root_outputs, int32_t* const* num_leaves_out);

/* Launch policy of a group, chosen by timing whole group iterations (GB300-only, no reference
 * counterpart; results never depend on it): for every member the same budget of histogram CTAs
 * (38, 19, 10 or 5 over all its feature tiles, with at least 1024, 2048, 4096 or 8192 rows each)
 * and partition CTAs (64, 32, 16 or 8), each with and without programmatic dependent launch — a
 * smaller budget lets more members' kernels run side by side. Every candidate runs one untimed and
 * `trials` timed iterations (median) on the given device gradients, without score updates; the
 * members' job states (their stochastic-rounding engines) are put back afterwards, so call it
 * before the first bk_learner_group_train. The fastest candidate is applied to every member
 * (bk_learner_set_launch_shape, bk_learner_set_launch_overlap) and written to policy_out (host,
 * 4 ints, may be NULL): {launch overlap on, rows per histogram CTA, histogram CTAs per member,
 * partition CTAs}. */
int bk_learner_group_autotune(bk_learner_group* group, const float* const* gradients, const float* const* hessians,
                              int32_t trials, int32_t* policy_out);

int bk_learner_group_destroy(bk_learner_group* group);

/* Replaces SerialTreeLearner::add_prediction_to_score (serial.rs:1974-1990): for every job j
 * and every row r of leaf l of the last tree, score[j][r] += leaf_values[j][l].
 * score: [num_jobs][num_data] f64, host or device (on_device); leaf_values: host. */
int bk_learner_add_prediction_to_score(bk_learner* learner, const double* leaf_values, double* score,
                                       int32_t on_device);

/* The leaf of every row after the last tree (-1 outside the bagged rows) — the partition that
 * SerialTreeLearner keeps in `pub partition` (serial.rs:212). out: [num_jobs][num_data] host. */
int bk_learner_row_leaf(bk_learner* learner, int32_t* out);

/* Grow-loop execution: 0 = one host round trip per split (the plain form); 1 = the whole
 * grow loop of an iteration captured once as a CUDA graph and replayed (default). */
int bk_learner_set_loop_mode(bk_learner* learner, int32_t mode);

/* Grow-loop kernel launches: 1 (default) = each kernel is launched with programmatic dependent
 * launch, so it is scheduled while the previous kernel finishes; 0 = plain stream order. */
int bk_learner_set_launch_overlap(bk_learner* learner, int32_t on);

/* The by-tree column sample of the following train calls: the `is_feature_used_bytree` mask that
 * ColSampler::reset_by_tree draws before each tree (treelearner/col_sampler.rs:87-103) and
 * find_best_splits applies (serial.rs:839-854): features with mask 0 are neither searched nor
 * split on. mask: host uint8 [num_jobs][num_features] over inner features (one mask per class
 * tree, as the reference draws one per train call), or NULL for "every feature". */
int bk_learner_set_feature_mask(bk_learner* learner, const uint8_t* mask);

/* The by-node column sample (ColSampler::get_by_node, treelearner/col_sampler.rs:109-177, without
 * interaction constraints) of the following train calls: every searched leaf — the smaller one,
 * then the larger one, at every split — draws Random::sample(n, get_cnt(n, fraction)) of its
 * candidate features on the device, the candidates being the tree's by-tree sample (the
 * bk_learner_set_feature_mask mask) when bytree_active, else every feature; a leaf's best split
 * comes only from its sample (serial.rs:1328-1336, :1538-1554). rng_state is the sampler's LCG
 * state after the host's by-tree draw for the coming tree; the state after the tree's by-node
 * draws is read back with bk_learner_bynode_state, so the host's next by-tree draw continues the
 * same stream. fraction >= 1 turns it off. Needs num_jobs == 1 (the reference draws the K class
 * trees' samples from one stream, one tree after the other). */
int bk_learner_set_bynode(bk_learner* learner, double fraction, int32_t bytree_active, uint32_t rng_state);

/* The by-node sampler's LCG state after the last train call. */
int bk_learner_bynode_state(bk_learner* learner, uint32_t* rng_state);

/* Interaction constraints (config interaction_constraints; ColSampler::get_by_node's allowed
 * features, treelearner/col_sampler.rs:148-177): a searched leaf may split only on the features
 * on its path (serial.rs:1719-1722) and on those of every set that holds the whole path (every
 * set at the root); with by-node sampling the sample is drawn among the allowed features. Set k
 * holds the real feature indices features[offsets[k] .. offsets[k + 1]); num_sets 0 removes the
 * constraints. Applies to the following train calls. */
int bk_learner_set_interaction_constraints(bk_learner* learner, const int32_t* features, const int32_t* offsets,
                                           int32_t num_sets);

/* Launch-shape autotuner (GB300-only, no reference counterpart; results never depend on it).
 * Times whole trees (graph form, median of `trials` after one untimed tree per shape) grown from
 * the given gradients (as bk_learner_train takes them, all rows) over a coordinate descent of
 * five launch parameters — the fewest rows a histogram CTA takes, histogram CTAs per 32-feature
 * tile, partition CTAs, and (quantized) the most rows a histogram CTA adds straight to the pool
 * slot with global atomics instead of through a shared histogram, and the histogram CTAs of a tile
 * per thread-block cluster (1, 2 or 4; a cluster adds up its CTAs' shared histograms in distributed
 * shared memory before one flush) — and keeps the fastest. Choices are cached per shape class (device,
 * log2 rows, feature tiles, bins per feature, quantized, num_leaves, num_jobs): a later learner of
 * the same class takes the cached shape without timing. The learner's state across trees (the
 * stochastic-rounding engine) is restored afterwards; the trial trees replace the "last tree"
 * outputs (bk_learner_row_leaf), so call it before the first bk_learner_train. shape_out (host,
 * 5 ints, may be NULL) receives the chosen shape. */
int bk_learner_autotune(bk_learner* learner, const float* gradients, const float* hessians, int32_t on_device,
                        int32_t trials, int32_t* shape_out);

/* The current launch shape (5 ints): {rows per histogram CTA (minimum), histogram CTAs per
 * feature tile, partition CTAs, rows per histogram CTA up to which it uses global atomics (0:
 * never), histogram CTAs per cluster (1: none)}. */
int bk_learner_launch_shape(bk_learner* learner, int32_t* shape_out);

/* Sets the launch shape (e.g. one found by bk_learner_autotune earlier), clamped to what the
 * dataset's rows can fill: shape[0] >= 32 rows (rounded down to a multiple of 32), shape[1] >= 1,
 * shape[2] >= 1 (at most 1024), shape[3] >= 0 (used on the quantized path only), shape[4] in
 * 0 .. 8 (0 or 1: no cluster; 2, 3 -> 2; 4 .. 7 -> 4; 8; quantized path only; the histogram CTAs
 * per tile become a multiple of it). 5 ints. */
int bk_learner_set_launch_shape(bk_learner* learner, const int32_t* shape);

/* Replaces SerialTreeLearner::reset_constant_hessian (serial.rs:279). */
int bk_learner_reset_constant_hessian(bk_learner* learner, int32_t value);

/* Threads per split-search CTA (one CTA per leaf side and feature) of the learner's next train call
 * (GB300-only): 64 when every feature is numerical with at most 63 searched bins and the grow
 * loop runs the single-pass form without L1 / max_delta_step / path_smooth, else 256. */
int bk_learner_search_threads(bk_learner* learner, int32_t* threads);

/* Replaces SerialTreeLearner::histogram_cache_capacity (serial.rs:250-252): the histogram slots
 * the learner keeps, into *capacity (host). This learner always keeps a full pool, one slot per
 * leaf (num_leaves), whatever histogram_pool_size says; the pool size never changes a result. */
int bk_learner_histogram_cache_capacity(bk_learner* learner, int64_t* capacity);

/* Replaces SerialTreeLearner::reset_histogram_pool_config (serial.rs:254-264), the Trainer's
 * budget-only reset (boosting/train.rs:997-1003): the learner keeps its rows, its by-node
 * sampler's state and its pool (always full here), so the call changes nothing and only checks the
 * handle. The by-tree sample that the reference redraws there is the host's (it passes the mask
 * with bk_learner_set_feature_mask). */
int bk_learner_reset_histogram_pool_config(bk_learner* learner);

/* Timing of the last train call, from CUDA events on the learner's stream: total device time
 * and the histogram kernels' time (ms), plus the algorithmic bytes the histogram kernels moved. */
int bk_learner_last_timing(bk_learner* learner, double* total_ms, double* hist_ms, double* hist_bytes);

/* With timing on: the split-search and partition phases of the last train call (ms). */
int bk_learner_last_phase_timing(bk_learner* learner, double* search_ms, double* partition_ms);

/* With timing on: the phases of every grow-loop step of the last train call, out[3 * i + k] (ms)
 * for step i = 0 .. num_leaves - 2 and k = histogram, split search, partition (-1 where a step
 * did not run). Step i builds the histogram of the smaller child of split i - 1 (the root's at
 * i = 0), searches both children and partitions split i. */
int bk_learner_last_step_timing(bk_learner* learner, float* out);

/* Enables (1) or disables (0) CUDA-event timing of every grow-loop phase of a train call
 * (histogram, split search, partition), reported by bk_learner_last_timing and
 * bk_learner_last_phase_timing. */
int bk_learner_set_timing(bk_learner* learner, int32_t on);

/* The learner's own device gradient / hessian buffers ([num_jobs][num_data] f32). A caller that
 * computes gradients on the device may write them here and pass these pointers to
 * bk_learner_train with on_device = 1, which then copies nothing. */
int bk_learner_gradient_buffers(bk_learner* learner, float** gradients, float** hessians);

/* Gradients of a built-in objective on the device, written into the learner's gradient buffers
 * (next-step work of the reference's Trainer: objective/regression.rs:240-248 (kind 0, L2),
 * objective/binary.rs:71-90 (kind 1, binary, `sigmoid`), objective/multiclass.rs:68-90 (kind 2,
 * softmax over num_jobs classes)). score: device [num_jobs][num_data] f64; label: device f32.
 * Enqueued on the learner's stream, ordered before its next call. */
int bk_learner_objective_gradients(bk_learner* learner, int32_t kind, const double* score, const float* label,
                                   double sigmoid);

/* Weights of the device objectives (bk_learner_objective_gradients), kept until changed:
 * weights: device f32 [num_data] row weights (Metadata::weights), or NULL for none; read by every
 * later gradient call, so it must stay valid while the learner uses it (the caller owns it).
 * neg_label_weight / pos_label_weight: the binary objective's label weights of the negative and
 * positive class (BinaryLogloss::label_weights, objective/binary.rs:33-52, which the host derives
 * from is_unbalance or scale_pos_weight); 1 and 1 for neither. Operation order of the weighted
 * gradients: objective/regression.rs:321-329 (L2), binary.rs:71-90, multiclass.rs:68-90. The loss
 * of bk_learner_objective_loss stays unweighted. */
int bk_learner_set_objective_weights(bk_learner* learner, const float* weights, double neg_label_weight,
                                     double pos_label_weight);

/* Mean training loss (L2: squared error; binary / multiclass: log loss) of a device score,
 * returned in *out (host). */
int bk_learner_objective_loss(bk_learner* learner, int32_t kind, const double* score, const float* label,
                              double* out);

/* Adds one trained tree's output to the scores of binned rows on the device: the replay of
 * SerialTreeLearner::add_prediction_for_rows (serial.rs:2009-2041) for rows outside the training
 * partition (held-out / out-of-bag rows). The tree is given as the node arrays of
 * tree.rs:310-403 (left_child / right_child with ~leaf for leaves, split_feature_inner,
 * threshold_in_bin, decision_type with the categorical bit 1 and the default-left bit 2) plus
 * leaf_value [num_leaves], all host. cat_bins: host [num_leaves - 1][8] uint32, for each
 * categorical node the bitset of the bin-mapper bins that go left (bk_split.cat_bins; the
 * categories of Tree::split_categorical mapped to bins), may be NULL when no node is categorical.
 * bins: device uint8 [num_features][num_rows] stored bins of the rows, made with this learner's
 * bin mappers; score: device f64 [num_rows]. */
int bk_learner_predict_add(bk_learner* learner, int32_t num_leaves, const int32_t* left_child,
                           const int32_t* right_child, const int32_t* split_feature_inner,
                           const uint32_t* threshold_in_bin, const int8_t* decision_type, const uint32_t* cat_bins,
                           const double* leaf_value, const uint8_t* bins, int64_t num_rows, double* score);

/* The histogram of one leaf of the last tree, as the learner's histogram pool holds it after the
 * tree (serial.rs:80-162 HistogramPool, with FixHistogram and the parent-minus-child subtraction of
 * serial.rs:1407-1437 applied): the leaf's slot, group bins of every inner feature in feature
 * order (io/dataset.rs:35-76, one dense group per feature: 1 + num_bin - (most_freq_bin == 0)
 * bins each). out: host [total group bins][2] (gradient, hessian) sums — double on the float
 * path, int64 on the quantized path (integer gradient / hessian units, unscaled). slot_out (may be
 * NULL): the pool slot, -1 when the leaf has none (it was never searched: -1 is returned). The
 * reference has no such call (its pool is private); it exists so a host can report the device
 * histograms' error against an f64 CPU learner. */
int bk_learner_leaf_histogram(bk_learner* learner, int32_t job, int32_t leaf, void* out, int32_t* slot_out);

/* The CUDA stream (cudaStream_t) every call of this learner is ordered on, for callers that
 * time or order their own work against the learner's. */
int bk_learner_stream(bk_learner* learner, void** stream);

int bk_learner_destroy(bk_learner* learner);

/* Stable partition of one row range, for callers that cannot allocate device memory (a host
 * whose GPU memory belongs to its own caching allocator, or a latency-critical path that cannot
 * take cudaMalloc's implicit synchronization). No counterpart in the reference: it is the
 * learner's DataPartition::Split kernel pair made callable on its own, with no allocation.
 * rows_in: device int32 row ids [num_rows]; bins: device uint8 stored bins indexed by row id
 * (bins_len entries); route: host uint8[256], route[b] != 0 sends stored bin b left; rows_out:
 * device int32 [num_rows], not aliasing rows_in, receives the left rows then the right rows, each
 * in input order; *num_left (host) receives the left count. stream: a cudaStream_t or NULL.
 * Synchronous. Its only scratch is a fixed 8 KiB device array inside the library (at most 2^30
 * rows; larger inputs are rejected), set up on the first call on each device — make that first
 * call before any stream capture. Calls that overlap on the GPU share that array and race. */
int bk_partition_split_noalloc(const int32_t* rows_in, int64_t num_rows, const uint8_t* bins, int64_t bins_len,
                               const uint8_t* route, int32_t* rows_out, int64_t* num_left, void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* bk_last_error(void);

/* ---- host-side dataset preparation (the reference's host keeps these, io/bin.rs) ---- */

/* BinMapper::find_bin for a numerical feature (io/bin.rs:342-554). */
int32_t bk_find_bin_numerical(double* values, int64_t num_values, int64_t total_sample_cnt, int32_t max_bin,
                              int32_t min_data_in_bin, int32_t min_split_data, int32_t pre_filter,
                              int32_t use_missing, int32_t zero_as_missing, double* upper_bounds, int32_t cap,
                              int32_t* meta_out, double* dmeta_out);

/* Stored group bins of one column (io/dataset.rs:633-685 with BinMapper::value_to_bin). */
void bk_values_to_group_bins(const double* col, int64_t n, int64_t stride, const double* upper_bounds,
                             int32_t num_bin, int32_t missing_type, int32_t most_freq_bin, uint8_t* out);

/* BinMapper::find_bin for a categorical feature (io/bin.rs:459-554): bin_to_category receives the
 * category code of every bin (bin 0 = -1, "other / missing"). */
int32_t bk_find_bin_categorical(double* values, int64_t num_values, int64_t total_sample_cnt, int32_t max_bin,
                                int32_t min_data_in_bin, int32_t min_split_data, int32_t pre_filter,
                                int32_t use_missing, int32_t zero_as_missing, int32_t* bin_to_category, int32_t cap,
                                int32_t* meta_out, double* dmeta_out);

/* Stored group bins of one categorical column (io/dataset.rs:633-685 with the categorical
 * BinMapper::value_to_bin, io/bin.rs:558-589). */
void bk_values_to_group_bins_categorical(const double* col, int64_t n, int64_t stride, const int32_t* bin_to_category,
                                         int32_t num_bin, int32_t most_freq_bin, uint8_t* out);

#ifdef __cplusplus
}
#endif

#endif /* BKGPU_H */

// Host side of the GB300 learner and the C ABI declared in include/bkgpu.h.
//
// One bk_learner owns one dataset resident in HBM and grows `num_jobs` trees per train call.
// The grow loop (serial.rs:578-628) runs on the device: every step of an iteration —
// histogram of the smaller leaf, split search of both children, arg-max leaf, partition,
// bookkeeping — is a kernel that reads its operands from the per-job JobState in device memory.
// Loop mode 0 launches the steps split by split and reads the stop flags back after each
// arg-max (the plain form, one host round trip per split); loop mode 1 captures the whole
// iteration (num_leaves - 1 steps) once as a CUDA graph and replays it, with the remaining steps
// of a finished tree returning at their first instruction.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bk_common.cuh"

using namespace bk;

namespace {

thread_local std::string g_last_error;

}  // namespace

// Shared with the other translation units of the library (bk_common.cuh).
void bk_set_last_error(const char* msg) { g_last_error = msg; }

namespace {

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

struct CudaError {
  std::string msg;
};

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) throw CudaError{std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

// ---- host std::mt19937 for the per-row stochastic-rounding noise (mt19937.rs:32-101) ----
struct HostMt {
  uint32_t st[624];
  int idx;
  explicit HostMt(uint32_t seed) {
    st[0] = seed;
    for (int i = 1; i < 624; ++i) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
    idx = 624;
  }
  uint32_t next() {
    if (idx >= 624) {
      for (int i = 0; i < 624; ++i) {
        uint32_t y = (st[i] & 0x80000000u) | (st[(i + 1) % 624] & 0x7fffffffu);
        uint32_t nx = st[(i + 397) % 624] ^ (y >> 1);
        if (y & 1u) nx ^= 0x9908b0dfu;
        st[i] = nx;
      }
      idx = 0;
    }
    uint32_t y = st[idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  double canonical() {  // libc++ generate_canonical<double, 53>
    double g1 = (double)next();
    double g2 = (double)next();
    double rp = 4294967296.0;
    double sp = g1 + g2 * rp;
    return sp / (rp * rp);
  }
};

// The two row-tiled copies of the column-major bins: rt [n][rt_stride] and tm, tile t's block
// [n][width_t] at tiles[t].tm_off; a 4-bit tile packs feature 2k into the low nibble of byte k
// and feature 2k + 1 into its high nibble; a 16-byte 8-bit tile holds the tile's first 16 features.
__global__ void k_pack_rowtile(const uint8_t* __restrict__ cm, uint8_t* __restrict__ rt, uint8_t* __restrict__ tm,
                               int64_t n, int F, int T, const TileGeom* __restrict__ tiles, int rt_stride) {
  int64_t total = n * T;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    int64_t tile = k / n, row = k % n;
    const TileGeom g = tiles[tile];
    uint32_t w[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      uint32_t v = 0;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        if (g.nibble) {  // byte q * 4 + b of the 16-byte run holds features 2 (q * 4 + b) and + 1
          const int f0 = (int)tile * TILE + 2 * (q * 4 + b);
          uint32_t lo = (q < 4 && f0 < F) ? cm[(size_t)f0 * n + row] : 0u;
          uint32_t hi = (q < 4 && f0 + 1 < F) ? cm[(size_t)(f0 + 1) * n + row] : 0u;
          v |= ((lo & 15u) | ((hi & 15u) << 4)) << (8 * b);
        } else {
          int f = (int)tile * TILE + q * 4 + b;
          uint32_t x = f < F ? cm[(size_t)f * n + row] : 0u;
          v |= x << (8 * b);
        }
      }
      w[q] = v;
    }
    uint4* dst = reinterpret_cast<uint4*>(rt + (size_t)row * rt_stride + g.rt_off);
    uint4* dtm = reinterpret_cast<uint4*>(tm + g.tm_off + (size_t)row * tile_width(g));
    dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
    dtm[0] = make_uint4(w[0], w[1], w[2], w[3]);
    if (g.width == 32) {
      dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
      dtm[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
  }
}

}  // namespace

struct bk_learner {
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  Params p{};
  int K = 1;
  int loop_mode = 1;
  bool timing = false;
  bool bynode_sampling = false;  // bk_learner_set_bynode with a fraction below 1
  int exact_quant_root = 1;
  HistLaunch hl{};
  // dataset
  DevFeature* d_feat = nullptr;
  std::vector<DevFeature> h_feat;
  uint8_t* d_bins_cm = nullptr;
  uint8_t* d_bins_rt = nullptr;  // [n][rt_stride]: gathered leaves
  uint8_t* d_bins_tm = nullptr;  // per tile [n][width]: the root and dense leaves
  std::vector<TileGeom> h_tiles;
  double* d_noise_g = nullptr;
  double* d_noise_h = nullptr;
  // jobs
  std::vector<Job> jobs;
  Job* d_jobs = nullptr;
  float* d_g = nullptr;
  float* d_h = nullptr;
  int32_t* d_rows = nullptr;
  size_t pool_bytes_per_job = 0;
  void* d_pool = nullptr;
  std::vector<void*> allocs;
  // host staging
  bk_split* h_records = nullptr;
  double* h_leaf_values = nullptr;
  JobState* h_state = nullptr;
  int32_t* d_bad_label = nullptr;  // multiclass labels outside [0, K) seen by the objective kernels
  ObjectiveWeights obj_w;          // row / label weights of the device objectives (caller-owned rows)
  int32_t* h_bad_label = nullptr;  // pinned copy, read by the train call that follows the gradients
  double* d_leaf_vals_in = nullptr;
  int32_t* d_tree = nullptr;     // one tree's node arrays for prediction (13 x (num_leaves - 1))
  double* d_tree_values = nullptr;
  std::vector<int32_t> h_tree;
  // graph
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_gen = 0;  // bumped whenever the captured kernels' parameters change

  // The captured grow loop no longer matches the learner's parameters: captured anew when next
  // needed (here and in every learner group that holds this learner).
  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    ++graph_gen;
  }
  // timing
  cudaEvent_t ev_start = nullptr, ev_end = nullptr;
  std::vector<cudaEvent_t> hist_events;
  double last_total_ms = 0, last_hist_ms = 0, last_hist_bytes = 0, last_search_ms = 0, last_part_ms = 0;

  template <typename T>
  T* dalloc(size_t count) {
    void* ptr = nullptr;
    CK(cudaMalloc(&ptr, std::max<size_t>(count * sizeof(T), 16)));
    allocs.push_back(ptr);
    return reinterpret_cast<T*>(ptr);
  }

  ~bk_learner() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (void* a : allocs) cudaFree(a);
    if (h_records) cudaFreeHost(h_records);
    if (h_leaf_values) cudaFreeHost(h_leaf_values);
    if (h_state) cudaFreeHost(h_state);
    if (h_bad_label) cudaFreeHost(h_bad_label);
    for (cudaEvent_t e : hist_events) cudaEventDestroy(e);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_end) cudaEventDestroy(ev_end);
    if (stream) cudaStreamDestroy(stream);
  }

  // The launch shape of the grow-loop kernels, clamped to what the dataset's rows can fill: a
  // leaf never has more rows than the dataset, so CTAs past n / min_rows would never get rows.
  // Results do not depend on it (integer histograms are exact; the float path changes only its
  // rounding order; the partitions it feeds are the same). The graph is captured anew.
  void set_launch_shape(int hist_min_rows, int hist_ctas_per_tile, int part_grid, int direct_rows, int cluster) {
    const int64_t n = p.n;
    hl.direct_rows = std::max(0, direct_rows);
    p.hist_min_rows = std::max(32, hist_min_rows / 32 * 32);
    hl.blocks_per_tile = (int)std::max<int64_t>(
        1, std::min<int64_t>(hist_ctas_per_tile, (n + p.hist_min_rows - 1) / p.hist_min_rows));
    // a cluster of 2, 4 or 8 CTAs of one tile (quantized path): the tile's CTAs a multiple of it
    hl.cluster = 1;
    if (p.quant && cluster >= 2) {
      hl.cluster = cluster >= 8 ? 8 : (cluster >= 4 ? 4 : 2);
      hl.blocks_per_tile = std::max(hl.cluster, hl.blocks_per_tile / hl.cluster * hl.cluster);
    }
    p.part_grid = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(part_grid, kMaxPartGrid), (n + 255) / 256));
    drop_graph();
  }

  void shape_of(int32_t* out) const {
    out[0] = p.hist_min_rows;
    out[1] = hl.blocks_per_tile;
    out[2] = p.part_grid;
    out[3] = hl.direct_rows;
    out[4] = hl.cluster;
  }

  bool capturing = false;
  void record_hist_event(int i) {
    if (!timing || (size_t)i >= hist_events.size()) return;
    // inside stream capture only an external record becomes a timed event node of the graph
    if (capturing) CK(cudaEventRecordWithFlags(hist_events[i], stream, cudaEventRecordExternal));
    else CK(cudaEventRecord(hist_events[i], stream));
  }

  // One grow-loop step (iteration `it`) of all jobs; with timing on, events split the step into
  // histogram / search / partition phases.
  // The plain form keeps the reference's stable compaction; so does leaf renewal, whose f64 sums
  // run in leaf row order. Otherwise split `it` is partitioned in one pass, counting into the
  // counter pair it & 1, and the histogram launch of step it + 1 applies its bookkeeping.
  bool stable_partition() const { return loop_mode == 0 || (p.quant && p.renew); }
  void step_a(int it) {
    const bool stable = stable_partition();
    record_hist_event(4 * it);
    launch_hist(jobs.data(), K, p, d_bins_rt, d_bins_tm, hl, !stable && it > 0, (it + 1) & 1, stream);
    record_hist_event(4 * it + 1);
    // it clears the counter pair that split it + 1 uses; on the stable path its last CTA also
    // decides the split, otherwise the partition does
    launch_search(jobs.data(), K, p, d_feat, stable ? -1 : (it + 1) & 1, stable, !stable && it > 0, stream);
    record_hist_event(4 * it + 2);
  }
  void step_b(int it) {
    const bool stable = stable_partition();
    launch_partition(jobs.data(), K, p, d_bins_cm, d_feat, stable, it & 1, !stable, stream);
    record_hist_event(4 * it + 3);
  }

  void tree_prologue() {
    launch_init_rows(d_jobs, K, p, d_rows, stream);
    if (p.quant) launch_discretize(d_jobs, K, p, d_noise_g, d_noise_h, stream);
    launch_root_sums(d_jobs, K, p, exact_quant_root, stream);
    CK(cudaMemsetAsync(d_pool, 0, pool_bytes_per_job * K, stream));
    launch_tree_begin(d_jobs, K, p, stream);
  }

  void tree_epilogue() {
    if (!stable_partition()) launch_apply_split(jobs.data(), K, p, (p.num_leaves - 2) & 1, stream);
    if (p.quant && p.renew) launch_renew(d_jobs, K, p, stream);
  }

  void run_graph() {
    if (!graph_exec) {
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      capturing = true;
      try {
        tree_prologue();
        for (int it = 0; it < p.num_leaves - 1; ++it) {
          step_a(it);
          step_b(it);
        }
        tree_epilogue();
      } catch (...) {
        capturing = false;
        cudaStreamEndCapture(stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      capturing = false;
      CK(cudaStreamEndCapture(stream, &g));
      CK(cudaGraphInstantiate(&graph_exec, g, 0));
      CK(cudaGraphDestroy(g));
    }
    CK(cudaGraphLaunch(graph_exec, stream));
  }

  void run_stepwise() {
    tree_prologue();
    for (int it = 0; it < p.num_leaves - 1; ++it) {
      step_a(it);
      // one host round trip per split: has every job stopped?
      for (int j = 0; j < K; ++j)
        CK(cudaMemcpyAsync(&h_state[j].stop, &jobs[j].st->stop, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
      CK(cudaStreamSynchronize(stream));
      bool all = true;
      for (int j = 0; j < K; ++j) all = all && h_state[j].stop;
      if (all) break;
      step_b(it);
    }
    tree_epilogue();
  }
};

namespace {

int fail_cuda(const CudaError& e) {
  set_error("CUDA error: %s", e.msg.c_str());
  return -1;
}

}  // namespace

extern "C" {

const char* bk_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"

namespace {

int learner_create(const bk_feature* features, int32_t num_features, const uint8_t* bins, int64_t num_data,
                   const bk_config* c, int32_t num_jobs, bk_learner** out, bool device_bins) {
  if (!features || !bins || !c || !out || num_features <= 0 || num_data <= 0 || num_jobs <= 0) {
    set_error("bk_learner_create: invalid arguments");
    return -1;
  }
  if (c->num_leaves < 2) {
    set_error("num_leaves must be at least 2");
    return -1;
  }
  if (num_data >= (int64_t)INT32_MAX) {
    set_error("num_data must fit in int32 row indices");
    return -1;
  }
  bool quant = c->use_quantized_grad && c->num_grad_quant_bins >= 2 && c->num_grad_quant_bins <= 127;
  if (quant) {
    // the device's integer histograms and prefix sums hold (grad << 32) + hess: every partial sum
    // of a leaf's gradients must fit in 32 signed bits and of its hessians in 32 unsigned bits
    const double max_g = c->num_grad_quant_bins / 2 + 1;
    const double max_h = c->is_constant_hessian ? 1 : c->num_grad_quant_bins;
    if ((double)num_data * max_g >= 2147483648.0 || (double)num_data * max_h >= 4294967296.0) {
      set_error("quantized histograms of %lld rows with %d gradient bins overflow 32-bit sums",
                (long long)num_data, c->num_grad_quant_bins);
      return -1;
    }
  }
  bk_learner* L = new bk_learner();
  try {
    CK(cudaGetDevice(&L->device));
    CK(cudaDeviceGetAttribute(&L->num_sms, cudaDevAttrMultiProcessorCount, L->device));
    CK(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
    Params& p = L->p;
    p.l1 = c->lambda_l1;
    p.l2 = c->lambda_l2;
    p.max_delta = c->max_delta_step;
    p.smooth = c->path_smooth;
    p.min_hess = c->min_sum_hessian_in_leaf;
    p.min_gain = c->min_gain_to_split;
    p.min_data = c->min_data_in_leaf;
    p.fused = c->fused_madd ? 1 : 0;
    p.use_l1 = c->lambda_l1 > 0.0;
    p.use_max = c->max_delta_step > 0.0;
    p.use_smooth = c->path_smooth > BK_EPS;
    p.quant = quant ? 1 : 0;
    p.pdl = 1;
    p.const_hess = c->is_constant_hessian ? 1 : 0;
    p.num_leaves = c->num_leaves;
    p.max_depth = c->max_depth;
    p.F = num_features;
    p.T = (num_features + TILE - 1) / TILE;
    p.quant_bins = c->num_grad_quant_bins;
    p.stochastic = c->stochastic_rounding ? 1 : 0;
    p.renew = c->quant_train_renew_leaf ? 1 : 0;
    p.n = num_data;
    p.cat_smooth = c->cat_smooth;
    p.cat_l2 = c->cat_l2;
    p.max_cat_threshold = c->max_cat_threshold;
    p.max_cat_to_onehot = c->max_cat_to_onehot;
    p.min_data_per_group = c->min_data_per_group;
    p.bynode = 0;
    p.n_icons = 0;
    p.path_words = (num_features + 31) / 32;
    p.icons = nullptr;
    L->K = num_jobs;
    int maxb = 0;
    for (int f = 0; f < num_features; ++f) {
      DevFeature d{};
      d.num_bin = features[f].num_bin;
      d.missing = features[f].missing_type;
      d.default_bin = features[f].default_bin;
      d.mfb = features[f].most_freq_bin;
      d.offset = d.mfb == 0 ? 1 : 0;
      d.gbins = 1 + d.num_bin - d.offset;
      d.real = features[f].real_feature;
      d.len = d.num_bin - d.offset;
      d.penalty = features[f].penalty;
      d.cat = features[f].bin_type == 1 ? 1 : 0;
      if (d.num_bin < 1 || d.gbins > 256 || d.missing < 0 || d.missing > 2 || d.mfb < 0 || d.mfb >= d.num_bin ||
          d.default_bin < 0 || d.default_bin >= d.num_bin) {
        set_error("feature %d: unsupported bin mapper (num_bin %d, missing %d, mfb %d, default %d)", f, d.num_bin,
                  d.missing, d.mfb, d.default_bin);
        delete L;
        return -1;
      }
      maxb = std::max(maxb, d.gbins);
      L->h_feat.push_back(d);
    }
    // Validate the stored bins once, as the reference's BinsCheck does (histogram.rs:50-65);
    // device-resident bins are checked on the device after the copy below.
    for (int f = 0; !device_bins && f < num_features; ++f) {
      const uint8_t* col = bins + (size_t)f * (size_t)num_data;
      int gb = L->h_feat[f].gbins;
      for (int64_t i = 0; i < num_data; ++i)
        if (col[i] >= gb) {
          set_error("feature %d row %lld: stored bin %d outside [0, %d)", f, (long long)i, (int)col[i], gb);
          delete L;
          return -1;
        }
    }
    p.B = (maxb + 7) / 8 * 8;
    // the plain single-pass search runs in 64-thread CTAs when every feature is numerical and its
    // searched slice has at most 63 bins (thread 63 holds the forward scan's position -1)
    p.search_narrow = 1;
    for (const DevFeature& d : L->h_feat)
      if (d.cat || d.len > 63) p.search_narrow = 0;
    // the feature tiles' stored-bin layouts: 16-byte runs of 4-bit bins for tiles whose features
    // all have at most 16 group bins, 8-bit runs otherwise (16 bytes for a last tile of at most
    // 16 features, else 32); each tile's shared histogram holds its largest feature's group bins
    {
      int64_t off = 0;
      for (int t = 0; t < p.T; ++t) {
        TileGeom g{};
        int tb = 0;
        const int nf_tile = std::min(num_features, (t + 1) * TILE) - t * TILE;
        for (int f = t * TILE; f < t * TILE + nf_tile; ++f) tb = std::max(tb, L->h_feat[f].gbins);
        g.bins = (tb + 7) / 8 * 8;
        g.nibble = tb <= 16 ? 1 : 0;
        g.width = (g.nibble || nf_tile <= 16) ? 16 : 32;
        g.rt_off = off;
        g.tm_off = off * num_data;
        off += tile_width(g);
        L->h_tiles.push_back(g);
      }
      // a row of bins_rt starts on a 64-byte boundary: a gathered row then costs the fewest 64-byte
      // DRAM bursts (112 bytes at a 112-byte stride touch three bursts in three rows of four, two
      // at a 128-byte stride)
      p.rt_stride = (int32_t)((off + 63) / 64 * 64);
    }
    // launch shapes: histogram CTAs of 1024 threads, one per SM, split evenly over the feature
    // tiles, each taking at least 256 rows; two partition CTAs per SM; no more CTAs than the
    // dataset's rows can fill; no direct-atomic CTAs (bk_learner_autotune may change all four)
    L->hl.threads = 1024;
    L->set_launch_shape(256, L->num_sms / p.T, 2 * L->num_sms, 0, 1);
    bool wide = false;
    if (quant) {
      int max_h = p.const_hess ? 1 : p.quant_bins;
      int max_g = p.quant_bins / 2 + 1;
      int flush_rows = std::min(65535 / max_h, 32767 / max_g);
      int per_round = 32 * (L->hl.threads / 32);
      L->hl.flush_rounds = flush_rows / per_round;
      wide = L->hl.flush_rounds == 0;
      // the f64 root sums equal the sequential ones when every partial sum is exact
      bool pow2 = (p.quant_bins & (p.quant_bins - 1)) == 0;
      L->exact_quant_root = (pow2 && (double)num_data * (double)p.quant_bins < 536870912.0) ? 1 : 0;
    }
    L->hl.smem = hist_smem_bytes(p, L->hl.threads, quant, wide);
    if (L->hl.smem > 227 * 1024) {
      set_error("histogram tile needs %zu bytes of shared memory", L->hl.smem);
      delete L;
      return -1;
    }
    CK(hist_set_smem_attrs(L->hl.smem));

    const size_t n = (size_t)num_data;
    L->d_feat = L->dalloc<DevFeature>(num_features);
    CK(cudaMemcpy(L->d_feat, L->h_feat.data(), sizeof(DevFeature) * num_features, cudaMemcpyHostToDevice));
    L->d_bins_cm = L->dalloc<uint8_t>(n * num_features);
    CK(cudaMemcpy(L->d_bins_cm, bins, n * num_features, device_bins ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    if (device_bins) {
      int64_t bad = INT64_MAX;
      CK(check_bins_device(L->d_bins_cm, num_data, num_features, L->d_feat, &bad, L->stream));
      if (bad != INT64_MAX) {
        uint8_t v = 0;
        CK(cudaMemcpy(&v, L->d_bins_cm + bad, 1, cudaMemcpyDeviceToHost));
        const int f = (int)(bad / num_data);
        set_error("feature %d row %lld: stored bin %d outside [0, %d)", f, (long long)(bad % num_data), (int)v,
                  L->h_feat[f].gbins);
        delete L;
        return -1;
      }
    }
    TileGeom* d_tiles = L->dalloc<TileGeom>(p.T);
    CK(cudaMemcpy(d_tiles, L->h_tiles.data(), sizeof(TileGeom) * p.T, cudaMemcpyHostToDevice));
    p.tiles = d_tiles;
    L->d_bins_rt = L->dalloc<uint8_t>(n * (size_t)p.rt_stride);
    L->d_bins_tm = L->dalloc<uint8_t>(n * (size_t)p.rt_stride);
    k_pack_rowtile<<<4 * L->num_sms, 256, 0, L->stream>>>(L->d_bins_cm, L->d_bins_rt, L->d_bins_tm, num_data,
                                                          num_features, p.T, d_tiles, p.rt_stride);
    CK(cudaGetLastError());
    if (quant && p.stochastic) {
      // GradientDiscretizer::init_stochastic (gradient_discretizer/mod.rs:87-106)
      std::vector<double> ng(n), nh(n);
      size_t threads = (size_t)std::max(1, c->num_threads);
      size_t nb = std::min(threads, (n + 511) / 512), bs = n;
      if (nb > 1) bs = ((n + nb - 1) / nb + 31) / 32 * 32;
      if (nb < 1) nb = 1;
      for (size_t b = 0; b < nb; ++b) {
        size_t s0 = b * bs, s1 = std::min(s0 + bs, n);
        HostMt ge((uint32_t)c->seed + (uint32_t)b), he((uint32_t)c->seed + (uint32_t)b + (uint32_t)threads);
        for (size_t i = s0; i < s1; ++i) {
          ng[i] = ge.canonical();
          nh[i] = he.canonical();
        }
      }
      L->d_noise_g = L->dalloc<double>(n);
      L->d_noise_h = L->dalloc<double>(n);
      CK(cudaMemcpy(L->d_noise_g, ng.data(), n * sizeof(double), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(L->d_noise_h, nh.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    }
    const int Lv = p.num_leaves, F = num_features, K = num_jobs;
    L->d_g = L->dalloc<float>(n * K);
    L->d_h = L->dalloc<float>(n * K);
    L->d_rows = L->dalloc<int32_t>(n);
    L->pool_bytes_per_job = (size_t)Lv * p.T * p.B * TILE * (quant ? sizeof(int64_t) : sizeof(double2));
    L->d_pool = L->dalloc<uint8_t>(L->pool_bytes_per_job * K);
    JobState* d_states = L->dalloc<JobState>(K);
    CK(cudaMemset(d_states, 0, sizeof(JobState) * K));
    for (int j = 0; j < K; ++j) {  // no by-node sampling until bk_learner_set_bynode
      const double one = 1.0;
      CK(cudaMemcpy(&d_states[j].bynode_fraction, &one, sizeof(double), cudaMemcpyHostToDevice));
    }
    L->jobs.resize(K);
    for (int j = 0; j < K; ++j) {
      Job& J = L->jobs[j];
      J.st = d_states + j;
      J.g = L->d_g + (size_t)j * n;
      J.h = L->d_h + (size_t)j * n;
      J.packed = quant ? L->dalloc<int16_t>(n) : nullptr;
      J.idx0 = L->dalloc<int32_t>(n);
      J.idx1 = L->dalloc<int32_t>(n);
      J.pk0 = quant ? L->dalloc<int16_t>(n) : nullptr;
      J.pk1 = quant ? L->dalloc<int16_t>(n) : nullptr;
      J.leaf_begin = L->dalloc<int64_t>(Lv);
      J.leaf_count = L->dalloc<int64_t>(Lv);
      J.leaf_buf = L->dalloc<int32_t>(Lv);
      J.leaf_depth = L->dalloc<int32_t>(Lv);
      J.leaf_slot = L->dalloc<int32_t>(Lv);
      J.leaf_sum = L->dalloc<LeafSum>(Lv);
      J.bgain = L->dalloc<double>(Lv);
      J.bfeat = L->dalloc<int32_t>(Lv);
      // the candidates, then the categorical candidates' bin bitsets
      J.cand = L->dalloc<Cand>((size_t)Lv * F + (cand_cat_words(Lv, F) * sizeof(uint32_t) + sizeof(Cand) - 1) /
                                                     sizeof(Cand));
      J.cgain = L->dalloc<double>(2 * (size_t)F);
      J.csplit = L->dalloc<uint8_t>(2 * (size_t)F);
      J.cthr = L->dalloc<uint32_t>(2 * (size_t)F);
      J.bsplit = L->dalloc<int64_t>(Lv);
      J.lconst = L->dalloc<LeafConst>(2);
      J.splittable = L->dalloc<uint8_t>((size_t)Lv * F);
      // used, the two by-node masks, the sample scratch, then every leaf's path bitset
      J.used = L->dalloc<uint8_t>(4 * (size_t)F + sizeof(uint32_t) * (size_t)Lv * p.path_words);
      CK(cudaMemset(J.used, 1, 4 * (size_t)F));
      CK(cudaMemset(J.used + 4 * (size_t)F, 0, sizeof(uint32_t) * (size_t)Lv * p.path_words));
      J.tree_mask = L->dalloc<uint8_t>(F);
      CK(cudaMemset(J.tree_mask, 1, F));
      J.records = L->dalloc<bk_split>(Lv);
      J.leaf_value = L->dalloc<double>(Lv);
      J.pool = reinterpret_cast<uint8_t*>(L->d_pool) + L->pool_bytes_per_job * j;
      J.part_cnt = L->dalloc<int64_t>(kMaxPartGrid);
      J.red = L->dalloc<double>(2 * kRootGrid);
      J.ired = L->dalloc<int64_t>(2 * kRootGrid);
      CK(cudaMemset(J.records, 0, sizeof(bk_split) * Lv));
    }
    L->d_jobs = L->dalloc<Job>(K);
    CK(cudaMemcpy(L->d_jobs, L->jobs.data(), sizeof(Job) * K, cudaMemcpyHostToDevice));
    if (quant && p.stochastic) launch_mt_seed(L->d_jobs, K, (uint32_t)c->seed, L->stream);
    CK(cudaMallocHost(&L->h_records, sizeof(bk_split) * (size_t)Lv * K));
    CK(cudaMallocHost(&L->h_leaf_values, sizeof(double) * (size_t)Lv * K));
    CK(cudaMallocHost(&L->h_state, sizeof(JobState) * K));
    CK(cudaMallocHost(&L->h_bad_label, sizeof(int32_t)));
    *L->h_bad_label = 0;
    L->d_bad_label = L->dalloc<int32_t>(1);
    CK(cudaMemset(L->d_bad_label, 0, sizeof(int32_t)));
    L->d_leaf_vals_in = L->dalloc<double>((size_t)Lv * K);
    L->d_tree = L->dalloc<int32_t>(13 * (size_t)Lv);
    L->d_tree_values = L->dalloc<double>(Lv);
    CK(cudaEventCreate(&L->ev_start));
    CK(cudaEventCreate(&L->ev_end));
    CK(cudaStreamSynchronize(L->stream));
    CK(cudaGetLastError());
  } catch (const CudaError& e) {
    delete L;
    return fail_cuda(e);
  }
  *out = L;
  return 0;
}

}  // namespace

extern "C" {

int bk_learner_create(const bk_feature* features, int32_t num_features, const uint8_t* bins, int64_t num_data,
                      const bk_config* c, int32_t num_jobs, bk_learner** out) {
  return learner_create(features, num_features, bins, num_data, c, num_jobs, out, false);
}

int bk_learner_create_device_bins(const bk_feature* features, int32_t num_features, const uint8_t* bins,
                                  int64_t num_data, const bk_config* c, int32_t num_jobs, bk_learner** out) {
  return learner_create(features, num_features, bins, num_data, c, num_jobs, out, true);
}

namespace {

// The asynchronous half of a train call, all on the learner's stream: the gradient and row copies,
// the grow loop of every job, optionally the score update with the new trees (shrunk on the
// device), and the copies of the split records, leaf values and job states into pinned host
// buffers. Returns false with the error set on invalid arguments; CUDA errors throw.
bool train_enqueue(bk_learner* L, const float* gradients, const float* hessians, int32_t on_device,
                   const int32_t* rows, int64_t num_rows, double shrinkage, double* score) {
  const Params& p = L->p;
  const size_t n = (size_t)p.n, K = (size_t)L->K;
  const int Lv = p.num_leaves;
  if (rows && (num_rows <= 0 || num_rows > (int64_t)n)) {
    set_error("bk_learner_train: num_rows out of range");
    return false;
  }
  CK(cudaEventRecord(L->ev_start, L->stream));
  cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (gradients != L->d_g) CK(cudaMemcpyAsync(L->d_g, gradients, n * K * sizeof(float), kind, L->stream));
  if (hessians != L->d_h) CK(cudaMemcpyAsync(L->d_h, hessians, n * K * sizeof(float), kind, L->stream));
  int64_t root_count = rows ? num_rows : (int64_t)n;
  if (rows) CK(cudaMemcpyAsync(L->d_rows, rows, sizeof(int32_t) * num_rows, cudaMemcpyHostToDevice, L->stream));
  for (size_t j = 0; j < K; ++j) {
    L->h_state[j].use_rows = rows ? 1 : 0;
    L->h_state[j].root_count = root_count;
    L->h_state[j].hist_rows_direct = L->h_state[j].hist_rows_gather = L->h_state[j].hist_builds = 0;
    JobState* st = L->jobs[j].st;
    CK(cudaMemcpyAsync(&st->use_rows, &L->h_state[j].use_rows, sizeof(int32_t), cudaMemcpyHostToDevice,
                       L->stream));
    CK(cudaMemcpyAsync(&st->root_count, &L->h_state[j].root_count, sizeof(int64_t), cudaMemcpyHostToDevice,
                       L->stream));
    CK(cudaMemcpyAsync(&st->hist_rows_direct, &L->h_state[j].hist_rows_direct, 3 * sizeof(int64_t),
                       cudaMemcpyHostToDevice, L->stream));
  }
  if (L->timing && L->hist_events.size() != (size_t)(4 * (Lv - 1))) {
    for (cudaEvent_t e : L->hist_events) cudaEventDestroy(e);
    L->hist_events.assign(4 * (Lv - 1), nullptr);
    for (auto& e : L->hist_events) CK(cudaEventCreate(&e));
    L->drop_graph();
  }
  if (L->loop_mode == 1) L->run_graph();
  else L->run_stepwise();
  if (score) {
    launch_add_score_own(L->d_jobs, L->K, p, shrinkage, score, L->stream);
    CK(cudaGetLastError());
  }
  for (size_t j = 0; j < K; ++j) {
    const Job& J = L->jobs[j];
    CK(cudaMemcpyAsync(L->h_records + j * Lv, J.records, sizeof(bk_split) * (Lv - 1), cudaMemcpyDeviceToHost,
                       L->stream));
    CK(cudaMemcpyAsync(L->h_leaf_values + j * Lv, J.leaf_value, sizeof(double) * Lv, cudaMemcpyDeviceToHost,
                       L->stream));
    CK(cudaMemcpyAsync(&L->h_state[j], J.st, offsetof(JobState, mt), cudaMemcpyDeviceToHost, L->stream));
  }
  // labels the objective kernels rejected since the previous train call
  CK(cudaMemcpyAsync(L->h_bad_label, L->d_bad_label, sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
  CK(cudaMemsetAsync(L->d_bad_label, 0, sizeof(int32_t), L->stream));
  CK(cudaEventRecord(L->ev_end, L->stream));
  return true;
}

// After train_finish: a multiclass label outside [0, K) met by bk_learner_objective_gradients
// before this train call fails the call (the trees were grown on those gradients).
bool labels_ok(bk_learner* L) {
  if (*L->h_bad_label == 0) return true;
  set_error("bk_learner_objective_gradients: %d multiclass labels outside [0, %d) before this train call",
            *L->h_bad_label, L->K);
  return false;
}

// The synchronous half: waits for the learner's stream, reads the timings and fills the outputs.
void train_finish(bk_learner* L, bk_split* splits, double* leaf_values, double* root_outputs,
                  int32_t* num_leaves_out, bool timed = true) {
  const Params& p = L->p;
  const size_t K = (size_t)L->K;
  const int Lv = p.num_leaves;
  if (timed) {
    CK(cudaStreamSynchronize(L->stream));
    CK(cudaGetLastError());
  }
  float ms = 0.f;
  if (timed) CK(cudaEventElapsedTime(&ms, L->ev_start, L->ev_end));
  L->last_total_ms = ms;
  L->last_hist_ms = L->last_search_ms = L->last_part_ms = 0.0;
  if (L->timing && timed) {
    // the phases of the steps that ran (a finished tree's remaining steps return early but are
    // still timed: they are part of the replayed graph); a stepwise loop that stopped early
    // leaves later events unrecorded, which the elapsed-time calls report and skip
    for (int it = 0; it < Lv - 1; ++it) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, L->hist_events[4 * it], L->hist_events[4 * it + 1]) == cudaSuccess)
        L->last_hist_ms += t;
      if (cudaEventElapsedTime(&t, L->hist_events[4 * it + 1], L->hist_events[4 * it + 2]) == cudaSuccess)
        L->last_search_ms += t;
      if (cudaEventElapsedTime(&t, L->hist_events[4 * it + 2], L->hist_events[4 * it + 3]) == cudaSuccess)
        L->last_part_ms += t;
    }
    cudaGetLastError();
  }
  double bytes = 0.0;
  for (size_t j = 0; j < K; ++j) {
    const JobState& s = L->h_state[j];
    double bin_bytes = 0.0;  // a 4-bit tile's features take half a byte each
    for (int f = 0; f < p.F; ++f) bin_bytes += L->h_tiles[f / TILE].nibble ? 0.5 : 1.0;
    double per_row = bin_bytes + (p.quant ? 2.0 : (p.const_hess ? 4.0 : 8.0));
    bytes += (double)s.hist_rows_direct * per_row + (double)s.hist_rows_gather * (per_row + 4.0);
    double slot_bytes = 0.0;
    for (const DevFeature& f : L->h_feat) slot_bytes += (double)f.gbins * (p.quant ? 8.0 : 16.0);
    bytes += (double)s.hist_builds * slot_bytes;
  }
  L->last_hist_bytes = bytes;
  for (size_t j = 0; j < K; ++j) {
    const JobState& s = L->h_state[j];
    int nl = s.tree_leaves;
    if (num_leaves_out) num_leaves_out[j] = nl;
    if (root_outputs) root_outputs[j] = s.root_output;
    if (splits) std::memcpy(splits + j * (Lv - 1), L->h_records + j * Lv, sizeof(bk_split) * (Lv - 1));
    if (leaf_values) std::memcpy(leaf_values + j * Lv, L->h_leaf_values + j * Lv, sizeof(double) * Lv);
  }
}

}  // namespace

int bk_learner_train(bk_learner* L, const float* gradients, const float* hessians, int32_t on_device,
                     const int32_t* rows, int64_t num_rows, bk_split* splits, double* leaf_values,
                     double* root_outputs, int32_t* num_leaves_out) {
  if (!L || !gradients || !hessians) {
    set_error("bk_learner_train: invalid arguments");
    return -1;
  }
  try {
    if (!train_enqueue(L, gradients, hessians, on_device, rows, num_rows, 0.0, nullptr)) return -1;
    train_finish(L, splits, leaf_values, root_outputs, num_leaves_out);
    if (!labels_ok(L)) return -1;
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

namespace {

// Autotuned launch shapes by shape class: (device, log2 rows, feature tiles, bins per feature
// slot, quantized, num_leaves, jobs) -> (hist_min_rows, hist CTAs per tile, partition CTAs).
std::mutex g_tune_mutex;
std::map<std::array<int, 7>, std::array<int, 5>> g_tune_cache;

std::array<int, 7> tune_key(const bk_learner* L) {
  int lg = 0;
  while ((int64_t(1) << (lg + 1)) <= L->p.n) ++lg;
  return {L->device, lg, L->p.T, L->p.B, L->p.quant, L->p.num_leaves, L->K};
}

}  // namespace

int bk_learner_autotune(bk_learner* L, const float* gradients, const float* hessians, int32_t on_device,
                        int32_t trials, int32_t* shape_out) {
  if (!L || !gradients || !hessians || trials < 1) {
    set_error("bk_learner_autotune: invalid arguments");
    return -1;
  }
  const auto key = tune_key(L);
  {
    std::lock_guard<std::mutex> g(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      L->set_launch_shape(it->second[0], it->second[1], it->second[2], it->second[3], it->second[4]);
      if (shape_out) L->shape_of(shape_out);
      return 0;
    }
  }
  const int sms = L->num_sms, T = L->p.T;
  const int saved_mode = L->loop_mode;
  JobState* saved = nullptr;
  const size_t state_bytes = sizeof(JobState) * (size_t)L->K;
  try {
    // the trial trees must not advance the learner's state across trees (the stochastic-rounding
    // engine): the job states are saved here and put back afterwards
    CK(cudaMallocAsync((void**)&saved, state_bytes, L->stream));
    CK(cudaMemcpyAsync(saved, L->jobs[0].st, state_bytes, cudaMemcpyDeviceToDevice, L->stream));
    const size_t n = (size_t)L->p.n * (size_t)L->K;
    cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (gradients != L->d_g) CK(cudaMemcpyAsync(L->d_g, gradients, n * sizeof(float), kind, L->stream));
    if (hessians != L->d_h) CK(cudaMemcpyAsync(L->d_h, hessians, n * sizeof(float), kind, L->stream));
    L->loop_mode = 1;
    std::map<std::array<int, 5>, double> seen;
    // one tree per trial (graph form) after one untimed tree of each shape; the median device time
    auto measure = [&](const std::array<int, 5>& c) -> std::pair<std::array<int, 5>, double> {
      L->set_launch_shape(c[0], c[1], c[2], c[3], c[4]);
      std::array<int, 5> s = {L->p.hist_min_rows, L->hl.blocks_per_tile, L->p.part_grid, L->hl.direct_rows,
                              L->hl.cluster};
      auto f = seen.find(s);
      if (f != seen.end()) return {s, f->second};
      std::vector<double> t;
      for (int r = 0; r <= trials; ++r) {
        CK(cudaMemcpyAsync(L->jobs[0].st, saved, state_bytes, cudaMemcpyDeviceToDevice, L->stream));
        if (!train_enqueue(L, L->d_g, L->d_h, 1, nullptr, 0, 0.0, nullptr)) throw CudaError{g_last_error};
        train_finish(L, nullptr, nullptr, nullptr, nullptr);
        if (r > 0) t.push_back(L->last_total_ms);
      }
      std::sort(t.begin(), t.end());
      seen[s] = t[t.size() / 2];
      return {s, t[t.size() / 2]};
    };
    // coordinate descent from the default shape: rows per histogram CTA, histogram CTAs per
    // feature tile, partition CTAs
    std::array<int, 5> best = {256, sms / T, 2 * sms, 0, 1};
    double best_ms = measure(best).second;
    auto consider = [&](std::array<int, 5> c) {
      auto r = measure(c);
      if (r.second < best_ms) {
        best_ms = r.second;
        best = c;
      }
    };
    // rows per histogram CTA: small values spread small leaves over more SMs; large ones give
    // mid-size leaves fewer CTAs, so fewer shared histograms to flush into the pool slot
    for (int mr : {64, 128, 512, 1024, 2048, 4096, 8192, 16384}) consider({mr, best[1], best[2], best[3], best[4]});
    for (int ct : {2 * sms / T, sms / (2 * T)}) consider({best[0], ct, best[2], best[3], best[4]});
    for (int pg : {sms, 4 * sms}) consider({best[0], best[1], pg, best[3], best[4]});
    if (L->p.quant) {
      // the global-atomic variant of the quantized histogram for CTAs with few rows
      for (int dr : {128, 256, 512, 1024, 2048}) consider({best[0], best[1], best[2], dr, best[4]});
      // clusters of a tile's CTAs that add up their histograms in distributed shared memory
      for (int cl : {2, 4}) consider({best[0], best[1], best[2], best[3], cl});
    }
    CK(cudaMemcpyAsync(L->jobs[0].st, saved, state_bytes, cudaMemcpyDeviceToDevice, L->stream));
    CK(cudaFreeAsync(saved, L->stream));
    saved = nullptr;
    CK(cudaStreamSynchronize(L->stream));
    L->loop_mode = saved_mode;
    L->set_launch_shape(best[0], best[1], best[2], best[3], best[4]);
    {
      std::lock_guard<std::mutex> g(g_tune_mutex);
      g_tune_cache[key] = best;
    }
    if (shape_out) L->shape_of(shape_out);
  } catch (const CudaError& e) {
    if (saved) {
      cudaMemcpyAsync(L->jobs[0].st, saved, state_bytes, cudaMemcpyDeviceToDevice, L->stream);
      cudaFreeAsync(saved, L->stream);
      cudaStreamSynchronize(L->stream);
    }
    L->loop_mode = saved_mode;
    set_error("bk_learner_autotune: %s", e.msg.c_str());
    return -1;
  }
  return 0;
}

int bk_learner_set_launch_shape(bk_learner* L, const int32_t* shape) {
  if (!L || !shape || shape[0] < 32 || shape[1] < 1 || shape[2] < 1 || shape[3] < 0 || shape[4] < 0 ||
      shape[4] > 8) {
    set_error("bk_learner_set_launch_shape: invalid arguments");
    return -1;
  }
  L->set_launch_shape(shape[0], shape[1], shape[2], shape[3], shape[4]);
  return 0;
}

int bk_learner_launch_shape(bk_learner* L, int32_t* shape_out) {
  if (!L || !shape_out) {
    set_error("bk_learner_launch_shape: invalid arguments");
    return -1;
  }
  L->shape_of(shape_out);
  return 0;
}

int bk_learners_train_batch(bk_learner* const* learners, int32_t count, const float* const* gradients,
                            const float* const* hessians, int32_t on_device, double shrinkage,
                            double* const* scores, bk_split* const* splits, double* const* leaf_values,
                            double* const* root_outputs, int32_t* const* num_leaves_out) {
  if (!learners || count <= 0 || !gradients || !hessians) {
    set_error("bk_learners_train_batch: invalid arguments");
    return -1;
  }
  for (int32_t i = 0; i < count; ++i) {
    if (!learners[i] || !gradients[i] || !hessians[i]) {
      set_error("bk_learners_train_batch: learner %d: invalid arguments", i);
      return -1;
    }
    for (int32_t k = 0; k < i; ++k)
      if (learners[k] == learners[i]) {
        set_error("bk_learners_train_batch: learner %d appears twice", i);
        return -1;
      }
  }
  int32_t i = 0;
  try {
    // every learner's iteration is queued on its own stream before any is waited for, so the
    // devices's schedulers interleave the independent grow loops
    for (i = 0; i < count; ++i)
      if (!train_enqueue(learners[i], gradients[i], hessians[i], on_device, nullptr, 0, shrinkage,
                         scores ? scores[i] : nullptr)) {
        std::string msg = "learner " + std::to_string(i) + ": " + g_last_error;
        for (int32_t k = 0; k < i; ++k) cudaStreamSynchronize(learners[k]->stream);
        set_error("bk_learners_train_batch: %s", msg.c_str());
        return -1;
      }
    for (i = 0; i < count; ++i)
      train_finish(learners[i], splits ? splits[i] : nullptr, leaf_values ? leaf_values[i] : nullptr,
                   root_outputs ? root_outputs[i] : nullptr, num_leaves_out ? num_leaves_out[i] : nullptr);
    for (i = 0; i < count; ++i)
      if (!labels_ok(learners[i])) {
        std::string msg = g_last_error;
        set_error("bk_learners_train_batch: learner %d: %s", i, msg.c_str());
        return -1;
      }
  } catch (const CudaError& e) {
    for (int32_t k = 0; k < count; ++k) cudaStreamSynchronize(learners[k]->stream);
    set_error("bk_learners_train_batch: learner %d: CUDA error: %s", i, e.msg.c_str());
    return -1;
  }
  return 0;
}


// ---- learner groups: many learners' iterations captured into one CUDA graph ----

namespace {

// One learner's share of a group iteration, issued into the group's capture on the learner's own
// stream: what train_enqueue issues for an iteration on device gradients (no bagging), the grow
// loop issued directly (it cannot launch its own graph inside another capture), and the score
// update and result readback.
void group_enqueue(bk_learner* L, const float* gradients, const float* hessians, double shrinkage, double* score) {
  const Params& p = L->p;
  const size_t n = (size_t)p.n, K = (size_t)L->K;
  const int Lv = p.num_leaves;
  if (gradients != L->d_g)
    CK(cudaMemcpyAsync(L->d_g, gradients, n * K * sizeof(float), cudaMemcpyDeviceToDevice, L->stream));
  if (hessians != L->d_h)
    CK(cudaMemcpyAsync(L->d_h, hessians, n * K * sizeof(float), cudaMemcpyDeviceToDevice, L->stream));
  for (size_t j = 0; j < K; ++j) {
    JobState* st = L->jobs[j].st;
    CK(cudaMemcpyAsync(&st->use_rows, &L->h_state[j].use_rows, sizeof(int32_t), cudaMemcpyHostToDevice, L->stream));
    CK(cudaMemcpyAsync(&st->root_count, &L->h_state[j].root_count, sizeof(int64_t), cudaMemcpyHostToDevice,
                       L->stream));
    CK(cudaMemcpyAsync(&st->hist_rows_direct, &L->h_state[j].hist_rows_direct, 3 * sizeof(int64_t),
                       cudaMemcpyHostToDevice, L->stream));
  }
  L->capturing = true;
  L->tree_prologue();
  for (int it = 0; it < Lv - 1; ++it) {
    L->step_a(it);
    L->step_b(it);
  }
  L->tree_epilogue();
  L->capturing = false;
  if (score) {
    launch_add_score_own(L->d_jobs, L->K, p, shrinkage, score, L->stream);
    CK(cudaGetLastError());
  }
  for (size_t j = 0; j < K; ++j) {
    const Job& J = L->jobs[j];
    CK(cudaMemcpyAsync(L->h_records + j * Lv, J.records, sizeof(bk_split) * (Lv - 1), cudaMemcpyDeviceToHost,
                       L->stream));
    CK(cudaMemcpyAsync(L->h_leaf_values + j * Lv, J.leaf_value, sizeof(double) * Lv, cudaMemcpyDeviceToHost,
                       L->stream));
    CK(cudaMemcpyAsync(&L->h_state[j], J.st, offsetof(JobState, mt), cudaMemcpyDeviceToHost, L->stream));
  }
  CK(cudaMemcpyAsync(L->h_bad_label, L->d_bad_label, sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
  CK(cudaMemsetAsync(L->d_bad_label, 0, sizeof(int32_t), L->stream));
}

}  // namespace

struct bk_learner_group {
  std::vector<bk_learner*> learners;
  std::vector<uint64_t> gens;     // each learner's graph generation when captured
  std::vector<const float*> g, h;  // the captured inputs
  std::vector<double*> scores;
  double shrinkage = 0.0;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t exec = nullptr;

  ~bk_learner_group() {
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (stream) cudaStreamDestroy(stream);
  }

  bool current(const float* const* gg, const float* const* hh, double shr, double* const* sc) const {
    if (!exec || shr != shrinkage) return false;
    for (size_t i = 0; i < learners.size(); ++i)
      if (gens[i] != learners[i]->graph_gen || g[i] != gg[i] || h[i] != hh[i] || scores[i] != (sc ? sc[i] : nullptr))
        return false;
    return true;
  }

  // Captures one iteration of every learner: a fork event on the group's stream, each learner's
  // stream joining the capture behind it, every learner's work on its own stream (independent
  // branches of one graph), and a join of every branch back into the group's stream.
  void capture(const float* const* gg, const float* const* hh, double shr, double* const* sc) {
    if (exec) {
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    try {
      CK(cudaEventRecord(fork, stream));
      for (size_t i = 0; i < learners.size(); ++i) {
        bk_learner* L = learners[i];
        CK(cudaStreamWaitEvent(L->stream, fork, 0));
        group_enqueue(L, gg[i], hh[i], shr, sc ? sc[i] : nullptr);
        CK(cudaEventRecord(joins[i], L->stream));
        CK(cudaStreamWaitEvent(stream, joins[i], 0));
      }
    } catch (...) {
      for (bk_learner* L : learners) L->capturing = false;
      cudaStreamEndCapture(stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    CK(cudaStreamEndCapture(stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(e);
    for (size_t i = 0; i < learners.size(); ++i) {
      gens[i] = learners[i]->graph_gen;
      g[i] = gg[i];
      h[i] = hh[i];
      scores[i] = sc ? sc[i] : nullptr;
    }
    shrinkage = shr;
  }
};

int bk_learner_group_create(bk_learner* const* learners, int32_t count, bk_learner_group** out) {
  if (!learners || count <= 0 || !out) {
    set_error("bk_learner_group_create: invalid arguments");
    return -1;
  }
  *out = nullptr;
  for (int32_t i = 0; i < count; ++i) {
    if (!learners[i]) {
      set_error("bk_learner_group_create: learner %d is null", i);
      return -1;
    }
    if (learners[i]->device != learners[0]->device) {
      set_error("bk_learner_group_create: learner %d is on device %d, learner 0 on device %d", i,
                learners[i]->device, learners[0]->device);
      return -1;
    }
    for (int32_t k = 0; k < i; ++k)
      if (learners[k] == learners[i]) {
        set_error("bk_learner_group_create: learner %d appears twice", i);
        return -1;
      }
  }
  auto G = std::make_unique<bk_learner_group>();
  try {
    G->device = learners[0]->device;
    CK(cudaSetDevice(G->device));
    G->learners.assign(learners, learners + count);
    G->gens.assign(count, 0);
    G->g.assign(count, nullptr);
    G->h.assign(count, nullptr);
    G->scores.assign(count, nullptr);
    CK(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&G->fork, cudaEventDisableTiming));
    G->joins.assign(count, nullptr);
    for (auto& e : G->joins) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  *out = G.release();
  return 0;
}

int bk_learner_group_train(bk_learner_group* G, const float* const* gradients, const float* const* hessians,
                           double shrinkage, double* const* scores, bk_split* const* splits,
                           double* const* leaf_values, double* const* root_outputs, int32_t* const* num_leaves_out) {
  if (!G || !gradients || !hessians) {
    set_error("bk_learner_group_train: invalid arguments");
    return -1;
  }
  const size_t count = G->learners.size();
  for (size_t i = 0; i < count; ++i) {
    const bk_learner* L = G->learners[i];
    if (!gradients[i] || !hessians[i]) {
      set_error("bk_learner_group_train: learner %d: null gradients", (int)i);
      return -1;
    }
    if (L->loop_mode != 1 || L->timing) {
      set_error("bk_learner_group_train: learner %d: a group runs the graph form without phase timing", (int)i);
      return -1;
    }
  }
  size_t i = 0;
  try {
    CK(cudaSetDevice(G->device));
    for (bk_learner* L : G->learners)
      for (int j = 0; j < L->K; ++j) {
        L->h_state[j].use_rows = 0;
        L->h_state[j].root_count = L->p.n;
        L->h_state[j].hist_rows_direct = L->h_state[j].hist_rows_gather = L->h_state[j].hist_builds = 0;
      }
    if (!G->current(gradients, hessians, shrinkage, scores)) G->capture(gradients, hessians, shrinkage, scores);
    // the iteration comes after the work already queued on every member's stream (the gradients
    // of bk_learner_objective_gradients, an earlier call)
    for (size_t k = 0; k < count; ++k) {
      CK(cudaEventRecord(G->joins[k], G->learners[k]->stream));
      CK(cudaStreamWaitEvent(G->stream, G->joins[k], 0));
    }
    CK(cudaGraphLaunch(G->exec, G->stream));
    CK(cudaStreamSynchronize(G->stream));
    CK(cudaGetLastError());
    for (i = 0; i < count; ++i)
      train_finish(G->learners[i], splits ? splits[i] : nullptr, leaf_values ? leaf_values[i] : nullptr,
                   root_outputs ? root_outputs[i] : nullptr, num_leaves_out ? num_leaves_out[i] : nullptr, false);
    for (i = 0; i < count; ++i)
      if (!labels_ok(G->learners[i])) {
        std::string msg = g_last_error;
        set_error("bk_learner_group_train: learner %d: %s", (int)i, msg.c_str());
        return -1;
      }
  } catch (const CudaError& e) {
    cudaStreamSynchronize(G->stream);
    set_error("bk_learner_group_train: CUDA error: %s", e.msg.c_str());
    return -1;
  }
  return 0;
}

int bk_learner_group_autotune(bk_learner_group* G, const float* const* gradients, const float* const* hessians,
                              int32_t trials, int32_t* policy_out) {
  if (!G || !gradients || !hessians || trials < 1) {
    set_error("bk_learner_group_autotune: invalid arguments");
    return -1;
  }
  const size_t count = G->learners.size();
  for (size_t i = 0; i < count; ++i)
    if (!gradients[i] || !hessians[i] || G->learners[i]->loop_mode != 1 || G->learners[i]->timing) {
      set_error("bk_learner_group_autotune: learner %d: null gradients, or not the graph form without timing", (int)i);
      return -1;
    }
  // (rows per histogram CTA at least, histogram CTAs per learner over all its tiles, partition CTAs):
  // from a quarter of the device per learner down to a thirtieth, so more learners' kernels run
  // side by side; each with and without programmatic dependent launch (whose early-resident CTAs
  // hold SM room that other learners' kernels could use)
  static const int kCand[4][3] = {{1024, 38, 64}, {2048, 19, 32}, {4096, 10, 16}, {8192, 5, 8}};
  std::vector<JobState*> saved(count, nullptr);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::vector<uint8_t> pdl0(count);
  std::vector<std::array<int, 5>> shape0(count);
  for (size_t i = 0; i < count; ++i) {
    pdl0[i] = (uint8_t)G->learners[i]->p.pdl;
    G->learners[i]->shape_of(shape0[i].data());
  }
  auto apply = [&](int pdl, int c) {
    for (bk_learner* L : G->learners) {
      if ((pdl != 0) != (L->p.pdl != 0)) {
        L->p.pdl = pdl;
        L->drop_graph();
      }
      L->set_launch_shape(kCand[c][0], std::max(1, kCand[c][1] / L->p.T), kCand[c][2], 0, 1);
    }
  };
  try {
    CK(cudaSetDevice(G->device));
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // the trial iterations must not advance the learners' state across trees (the stochastic-
    // rounding engines): every job state is saved here and put back before each trial and after
    for (size_t i = 0; i < count; ++i) {
      bk_learner* L = G->learners[i];
      CK(cudaMalloc((void**)&saved[i], sizeof(JobState) * (size_t)L->K));
      CK(cudaMemcpyAsync(saved[i], L->jobs[0].st, sizeof(JobState) * (size_t)L->K, cudaMemcpyDeviceToDevice,
                         L->stream));
    }
    for (bk_learner* L : G->learners) CK(cudaStreamSynchronize(L->stream));
    auto restore = [&]() {
      for (size_t i = 0; i < count; ++i)
        CK(cudaMemcpyAsync(G->learners[i]->jobs[0].st, saved[i], sizeof(JobState) * (size_t)G->learners[i]->K,
                           cudaMemcpyDeviceToDevice, G->stream));
    };
    double best_ms = 1e300;
    int best_pdl = 1, best_c = 0;
    for (int pdl = 1; pdl >= 0; --pdl)
      for (int c = 0; c < 4; ++c) {
        apply(pdl, c);
        for (bk_learner* L : G->learners)
          for (int j = 0; j < L->K; ++j) {
            L->h_state[j].use_rows = 0;
            L->h_state[j].root_count = L->p.n;
            L->h_state[j].hist_rows_direct = L->h_state[j].hist_rows_gather = L->h_state[j].hist_builds = 0;
          }
        G->capture(gradients, hessians, 0.0, nullptr);
        std::vector<float> t;
        for (int r = 0; r <= trials; ++r) {  // one untimed iteration, then `trials` timed ones
          restore();
          CK(cudaEventRecord(e0, G->stream));
          CK(cudaGraphLaunch(G->exec, G->stream));
          CK(cudaEventRecord(e1, G->stream));
          CK(cudaEventSynchronize(e1));
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, e0, e1));
          if (r > 0) t.push_back(ms);
        }
        std::sort(t.begin(), t.end());
        const double med = t[t.size() / 2];
        if (med < best_ms) {
          best_ms = med;
          best_pdl = pdl;
          best_c = c;
        }
      }
    restore();
    CK(cudaStreamSynchronize(G->stream));
    apply(best_pdl, best_c);
    if (policy_out) {
      policy_out[0] = best_pdl;
      policy_out[1] = kCand[best_c][0];
      policy_out[2] = kCand[best_c][1];
      policy_out[3] = kCand[best_c][2];
    }
  } catch (const CudaError& e) {
    cudaStreamSynchronize(G->stream);
    for (size_t i = 0; i < count; ++i) {
      bk_learner* L = G->learners[i];
      if (saved[i]) cudaMemcpy(L->jobs[0].st, saved[i], sizeof(JobState) * (size_t)L->K, cudaMemcpyDeviceToDevice);
      if ((pdl0[i] != 0) != (L->p.pdl != 0)) {
        L->p.pdl = pdl0[i];
        L->drop_graph();
      }
      L->set_launch_shape(shape0[i][0], shape0[i][1], shape0[i][2], shape0[i][3], shape0[i][4]);
    }
    for (JobState* x : saved) cudaFree(x);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    set_error("bk_learner_group_autotune: CUDA error: %s", e.msg.c_str());
    return -1;
  }
  for (JobState* x : saved) cudaFree(x);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

int bk_learner_group_destroy(bk_learner_group* G) {
  if (!G) return 0;
  cudaSetDevice(G->device);
  cudaStreamSynchronize(G->stream);
  delete G;
  return 0;
}

int bk_learner_add_prediction_to_score(bk_learner* L, const double* leaf_values, double* score, int32_t on_device) {
  if (!L || !leaf_values || !score) {
    set_error("bk_learner_add_prediction_to_score: invalid arguments");
    return -1;
  }
  const Params& p = L->p;
  const size_t n = (size_t)p.n, K = (size_t)L->K;
  try {
    CK(cudaMemcpyAsync(L->d_leaf_vals_in, leaf_values, sizeof(double) * p.num_leaves * K, cudaMemcpyHostToDevice,
                       L->stream));
    double* d_score = score;
    if (!on_device) {
      d_score = nullptr;
      CK(cudaMallocAsync((void**)&d_score, n * K * sizeof(double), L->stream));
      CK(cudaMemcpyAsync(d_score, score, n * K * sizeof(double), cudaMemcpyHostToDevice, L->stream));
    }
    launch_add_score(L->d_jobs, L->K, p, L->d_leaf_vals_in, d_score, L->stream);
    if (!on_device) {
      CK(cudaMemcpyAsync(score, d_score, n * K * sizeof(double), cudaMemcpyDeviceToHost, L->stream));
      CK(cudaFreeAsync(d_score, L->stream));
    }
    CK(cudaStreamSynchronize(L->stream));
    CK(cudaGetLastError());
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_row_leaf(bk_learner* L, int32_t* out) {
  if (!L || !out) {
    set_error("bk_learner_row_leaf: invalid arguments");
    return -1;
  }
  const Params& p = L->p;
  const size_t n = (size_t)p.n, K = (size_t)L->K;
  try {
    int32_t* d = nullptr;
    CK(cudaMallocAsync((void**)&d, n * K * sizeof(int32_t), L->stream));
    CK(cudaMemsetAsync(d, 0xff, n * K * sizeof(int32_t), L->stream));
    launch_row_leaf(L->d_jobs, L->K, p, d, L->stream);
    CK(cudaMemcpyAsync(out, d, n * K * sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
    CK(cudaFreeAsync(d, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    CK(cudaGetLastError());
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_set_loop_mode(bk_learner* L, int32_t mode) {
  if (!L || (mode != 0 && mode != 1)) {
    set_error("bk_learner_set_loop_mode: mode must be 0 or 1");
    return -1;
  }
  L->loop_mode = mode;
  return 0;
}

int bk_learner_set_launch_overlap(bk_learner* L, int32_t on) {
  if (!L) {
    set_error("bk_learner_set_launch_overlap: null learner");
    return -1;
  }
  if ((on != 0) != (L->p.pdl != 0)) L->drop_graph();
  L->p.pdl = on != 0;
  return 0;
}

int bk_learner_set_timing(bk_learner* L, int32_t on) {
  if (!L) {
    set_error("bk_learner_set_timing: null learner");
    return -1;
  }
  if ((on != 0) != L->timing) L->drop_graph();
  L->timing = on != 0;
  return 0;
}

int bk_learner_search_threads(bk_learner* L, int32_t* threads) {
  if (!L || !threads) {
    set_error("bk_learner_search_threads: invalid arguments");
    return -1;
  }
  const bool plain = !L->p.use_l1 && !L->p.use_max && !L->p.use_smooth;
  *threads = (plain && L->p.search_narrow && !L->stable_partition()) ? 64 : 256;
  return 0;
}

int bk_learner_histogram_cache_capacity(bk_learner* L, int64_t* capacity) {
  if (!L || !capacity) {
    set_error("bk_learner_histogram_cache_capacity: invalid arguments");
    return -1;
  }
  *capacity = L->p.num_leaves;  // a full pool: one slot per leaf
  return 0;
}

int bk_learner_reset_histogram_pool_config(bk_learner* L) {
  if (!L) {
    set_error("bk_learner_reset_histogram_pool_config: null learner");
    return -1;
  }
  return 0;
}

int bk_learner_reset_constant_hessian(bk_learner* L, int32_t value) {
  if (!L) {
    set_error("bk_learner_reset_constant_hessian: null learner");
    return -1;
  }
  if (L->p.quant) {
    set_error("constant-hessian changes after creation are not supported on the quantized path");
    return -1;
  }
  int v = value ? 1 : 0;
  if (v != L->p.const_hess) {
    L->p.const_hess = v;
    size_t smem = hist_smem_bytes(L->p, L->hl.threads, false, false);
    L->hl.smem = smem;
    cudaError_t e = hist_set_smem_attrs(smem);
    if (e != cudaSuccess) {
      set_error("CUDA error: %s", cudaGetErrorString(e));
      return -1;
    }
    L->drop_graph();
  }
  return 0;
}

int bk_learner_set_feature_mask(bk_learner* L, const uint8_t* mask) {
  if (!L) {
    set_error("bk_learner_set_feature_mask: null learner");
    return -1;
  }
  const size_t F = (size_t)L->p.F;
  try {
    for (int j = 0; j < L->K; ++j) {
      if (mask) {
        CK(cudaMemcpyAsync(L->jobs[j].tree_mask, mask + (size_t)j * F, F, cudaMemcpyHostToDevice, L->stream));
      } else {
        CK(cudaMemsetAsync(L->jobs[j].tree_mask, 1, F, L->stream));
      }
    }
    // the host mask may be freed or reused as soon as this call returns
    CK(cudaStreamSynchronize(L->stream));
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_set_bynode(bk_learner* L, double fraction, int32_t bytree_active, uint32_t rng_state) {
  if (!L) {
    set_error("bk_learner_set_bynode: null learner");
    return -1;
  }
  const bool on = fraction < 1.0;
  if (on && L->K != 1) {
    set_error("bk_learner_set_bynode: by-node sampling continues one sampler's stream across trees, which "
              "needs one tree per train call (num_jobs 1)");
    return -1;
  }
  if (on && !(fraction > 0.0)) {
    set_error("bk_learner_set_bynode: fraction must be in (0, 1]");
    return -1;
  }
  try {
    JobState* st = L->jobs[0].st;
    L->h_state[0].col_rng = rng_state;
    L->h_state[0].bytree_on = bytree_active ? 1 : 0;
    L->h_state[0].bynode_fraction = fraction;
    CK(cudaMemcpyAsync(&st->col_rng, &L->h_state[0].col_rng,
                       offsetof(JobState, bynode_fraction) + sizeof(double) - offsetof(JobState, col_rng),
                       cudaMemcpyHostToDevice, L->stream));
    CK(cudaStreamSynchronize(L->stream));
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  L->bynode_sampling = on;
  const int32_t masks = (on || L->p.n_icons > 0) ? 1 : 0;
  if (masks != L->p.bynode) L->drop_graph();
  L->p.bynode = masks;
  return 0;
}

int bk_learner_set_interaction_constraints(bk_learner* L, const int32_t* features, const int32_t* offsets,
                                           int32_t num_sets) {
  if (!L || num_sets < 0 || (num_sets > 0 && (!features || !offsets))) {
    set_error("bk_learner_set_interaction_constraints: invalid arguments");
    return -1;
  }
  const int W = L->p.path_words, F = L->p.F;
  std::vector<uint32_t> bits((size_t)num_sets * W, 0u);
  for (int32_t k = 0; k < num_sets; ++k) {
    if (offsets[k + 1] < offsets[k]) {
      set_error("bk_learner_set_interaction_constraints: offsets must not decrease");
      return -1;
    }
    for (int32_t i = offsets[k]; i < offsets[k + 1]; ++i)
      for (int f = 0; f < F; ++f)  // real feature -> inner feature; unused features drop out
        if (L->h_feat[f].real == features[i]) bits[(size_t)k * W + (f >> 5)] |= 1u << (f & 31);
  }
  try {
    const uint32_t* d = nullptr;
    if (num_sets > 0) {
      uint32_t* buf = L->dalloc<uint32_t>(bits.size());
      CK(cudaMemcpy(buf, bits.data(), sizeof(uint32_t) * bits.size(), cudaMemcpyHostToDevice));
      d = buf;
    }
    L->p.icons = d;
    L->p.n_icons = num_sets;
    L->p.bynode = (L->bynode_sampling || num_sets > 0) ? 1 : 0;
    L->drop_graph();  // the kernels take the constraints through their parameters
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_bynode_state(bk_learner* L, uint32_t* rng_state) {
  if (!L || !rng_state) {
    set_error("bk_learner_bynode_state: invalid arguments");
    return -1;
  }
  *rng_state = L->h_state[0].col_rng;  // copied back with the job state at the end of each train call
  return 0;
}

int bk_learner_last_timing(bk_learner* L, double* total_ms, double* hist_ms, double* hist_bytes) {
  if (!L) {
    set_error("bk_learner_last_timing: null learner");
    return -1;
  }
  if (total_ms) *total_ms = L->last_total_ms;
  if (hist_ms) *hist_ms = L->last_hist_ms;
  if (hist_bytes) *hist_bytes = L->last_hist_bytes;
  return 0;
}

int bk_learner_last_phase_timing(bk_learner* L, double* search_ms, double* partition_ms) {
  if (!L) {
    set_error("bk_learner_last_phase_timing: null learner");
    return -1;
  }
  if (search_ms) *search_ms = L->last_search_ms;
  if (partition_ms) *partition_ms = L->last_part_ms;
  return 0;
}

int bk_learner_last_step_timing(bk_learner* L, float* out) {
  if (!L || !out) {
    set_error("bk_learner_last_step_timing: invalid arguments");
    return -1;
  }
  if (!L->timing || L->hist_events.size() != (size_t)(4 * (L->p.num_leaves - 1))) {
    set_error("bk_learner_last_step_timing: timing is off (bk_learner_set_timing)");
    return -1;
  }
  for (int it = 0; it < L->p.num_leaves - 1; ++it)
    for (int k = 0; k < 3; ++k) {
      float t = -1.f;
      if (cudaEventElapsedTime(&t, L->hist_events[4 * it + k], L->hist_events[4 * it + k + 1]) != cudaSuccess)
        t = -1.f;
      out[3 * it + k] = t;
    }
  cudaGetLastError();  // an unrecorded event of a stepwise loop that stopped early is not an error
  return 0;
}

int bk_learner_gradient_buffers(bk_learner* L, float** gradients, float** hessians) {
  if (!L) {
    set_error("bk_learner_gradient_buffers: null learner");
    return -1;
  }
  if (gradients) *gradients = L->d_g;
  if (hessians) *hessians = L->d_h;
  return 0;
}

int bk_learner_objective_gradients(bk_learner* L, int32_t kind, const double* score, const float* label,
                                   double sigmoid) {
  if (!L || !score || !label || kind < 0 || kind > 2 || (kind == 2) != (L->K > 1) || L->K > 32) {
    set_error("bk_learner_objective_gradients: invalid arguments (kind %d, num_jobs %d)", kind, L ? L->K : 0);
    return -1;
  }
  try {
    CK(objective_gradients(kind, score, label, L->p.n, L->K, sigmoid, L->obj_w, L->d_g, L->d_h, L->d_bad_label,
                           L->stream));
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_set_objective_weights(bk_learner* L, const float* weights, double neg_label_weight,
                                     double pos_label_weight) {
  if (!L || !(neg_label_weight > 0.0) || !(pos_label_weight > 0.0) || std::isinf(neg_label_weight) ||
      std::isinf(pos_label_weight)) {
    set_error("bk_learner_set_objective_weights: invalid arguments");
    return -1;
  }
  L->obj_w.row = weights;
  L->obj_w.label_neg = neg_label_weight;
  L->obj_w.label_pos = pos_label_weight;
  return 0;
}

int bk_learner_objective_loss(bk_learner* L, int32_t kind, const double* score, const float* label, double* out) {
  if (!L || !score || !label || !out || kind < 0 || kind > 2 || (kind == 2) != (L->K > 1) || L->K > 32) {
    set_error("bk_learner_objective_loss: invalid arguments (kind %d, num_jobs %d)", kind, L ? L->K : 0);
    return -1;
  }
  try {
    const int grid = 512;
    double* d_part = L->jobs[0].red;  // 2 * kRootGrid >= grid doubles of scratch
    int32_t* d_bad = L->d_bad_label + 0;
    // the loss counts its own rejected labels: the gradients' count is kept for the next train call
    int32_t bad_before = 0, bad_after = 0;
    CK(cudaMemcpyAsync(&bad_before, d_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
    CK(objective_loss(kind, score, label, L->p.n, L->K, d_part, grid, d_bad, L->stream));
    std::vector<double> part(grid);
    CK(cudaMemcpyAsync(part.data(), d_part, sizeof(double) * grid, cudaMemcpyDeviceToHost, L->stream));
    CK(cudaMemcpyAsync(&bad_after, d_bad, sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    if (bad_after != bad_before) {
      CK(cudaMemcpy(d_bad, &bad_before, sizeof(int32_t), cudaMemcpyHostToDevice));
      set_error("bk_learner_objective_loss: %d multiclass labels outside [0, %d)", bad_after - bad_before, L->K);
      return -1;
    }
    double s = 0.0;
    for (double v : part) s += v;
    *out = s / (double)L->p.n;
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_predict_add(bk_learner* L, int32_t num_leaves, const int32_t* left_child, const int32_t* right_child,
                           const int32_t* split_feature_inner, const uint32_t* threshold_in_bin,
                           const int8_t* decision_type, const uint32_t* cat_bins, const double* leaf_value,
                           const uint8_t* bins, int64_t num_rows, double* score) {
  if (!L || !leaf_value || !bins || !score || num_rows < 0 || num_leaves < 1 || num_leaves > L->p.num_leaves ||
      (num_leaves > 1 && (!left_child || !right_child || !split_feature_inner || !threshold_in_bin ||
                          !decision_type))) {
    set_error("bk_learner_predict_add: invalid arguments");
    return -1;
  }
  const int ni = num_leaves - 1;
  // validate the node arrays so the device walk stays inside them
  for (int i = 0; i < ni; ++i) {
    for (int32_t ch : {left_child[i], right_child[i]}) {
      if (ch >= ni || (ch < 0 && ~ch >= num_leaves)) {
        set_error("bk_learner_predict_add: node %d has child %d outside the tree", i, ch);
        return -1;
      }
    }
    if (split_feature_inner[i] < 0 || split_feature_inner[i] >= L->p.F) {
      set_error("bk_learner_predict_add: node %d splits an unknown feature", i);
      return -1;
    }
    const bool cat = (decision_type[i] & 1) != 0;
    if (cat && (!cat_bins || !L->h_feat[split_feature_inner[i]].cat)) {
      set_error("bk_learner_predict_add: node %d is a categorical split without a bin bitset, or on a numerical "
                "feature", i);
      return -1;
    }
    if (!cat && threshold_in_bin[i] >= (uint32_t)L->h_feat[split_feature_inner[i]].num_bin) {
      set_error("bk_learner_predict_add: node %d splits an unknown feature or bin", i);
      return -1;
    }
  }
  L->h_tree.assign(13 * (size_t)std::max(ni, 1), 0);
  for (int i = 0; i < ni; ++i) {
    L->h_tree[i] = left_child[i];
    L->h_tree[ni + i] = right_child[i];
    L->h_tree[2 * ni + i] = split_feature_inner[i];
    L->h_tree[3 * ni + i] = (int32_t)threshold_in_bin[i];
    L->h_tree[4 * ni + i] = decision_type[i];
    if (decision_type[i] & 1)
      for (int w = 0; w < 8; ++w) L->h_tree[5 * ni + 8 * i + w] = (int32_t)cat_bins[8 * (size_t)i + w];
  }
  try {
    CK(cudaMemcpyAsync(L->d_tree, L->h_tree.data(), sizeof(int32_t) * L->h_tree.size(), cudaMemcpyHostToDevice,
                       L->stream));
    CK(cudaMemcpyAsync(L->d_tree_values, leaf_value, sizeof(double) * num_leaves, cudaMemcpyHostToDevice, L->stream));
    if (num_rows > 0)
      CK(predict_tree(L->d_feat, num_leaves, L->d_tree, L->d_tree_values, bins, num_rows, score, L->stream));
    CK(cudaStreamSynchronize(L->stream));
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_leaf_histogram(bk_learner* L, int32_t job, int32_t leaf, void* out, int32_t* slot_out) {
  if (!L || !out || job < 0 || job >= L->K || leaf < 0 || leaf >= L->p.num_leaves) {
    set_error("bk_learner_leaf_histogram: invalid arguments");
    return -1;
  }
  const Params& p = L->p;
  const Job& J = L->jobs[job];
  try {
    int32_t slot = -1;
    CK(cudaMemcpyAsync(&slot, J.leaf_slot + leaf, sizeof(int32_t), cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    if (slot_out) *slot_out = slot;
    if (slot < 0) {
      set_error("bk_learner_leaf_histogram: leaf %d of the last tree has no histogram", leaf);
      return -1;
    }
    // the slot [T][B][32]: tile f / 32, group bin b, lane f % 32
    const size_t cells = (size_t)p.T * p.B * TILE;
    const size_t elem = p.quant ? sizeof(int64_t) : sizeof(double2);
    std::vector<unsigned char> raw(cells * elem);
    CK(cudaMemcpyAsync(raw.data(), reinterpret_cast<const unsigned char*>(J.pool) + (size_t)slot * cells * elem,
                       cells * elem, cudaMemcpyDeviceToHost, L->stream));
    CK(cudaStreamSynchronize(L->stream));
    size_t o = 0;
    for (int f = 0; f < p.F; ++f) {
      const DevFeature& d = L->h_feat[f];
      for (int b = 0; b < d.gbins; ++b, ++o) {
        const size_t c = ((size_t)(f / TILE) * p.B + b) * TILE + (f % TILE);
        if (p.quant) {
          int64_t pk;
          std::memcpy(&pk, raw.data() + c * elem, sizeof(pk));
          const int64_t h = pk & 0xffffffffLL;
          reinterpret_cast<int64_t*>(out)[2 * o] = (pk - h) / 4294967296LL;
          reinterpret_cast<int64_t*>(out)[2 * o + 1] = h;
        } else {
          double2 v;
          std::memcpy(&v, raw.data() + c * elem, sizeof(v));
          reinterpret_cast<double*>(out)[2 * o] = v.x;
          reinterpret_cast<double*>(out)[2 * o + 1] = v.y;
        }
      }
    }
  } catch (const CudaError& e) {
    return fail_cuda(e);
  }
  return 0;
}

int bk_learner_stream(bk_learner* L, void** stream) {
  if (!L || !stream) {
    set_error("bk_learner_stream: invalid arguments");
    return -1;
  }
  *stream = (void*)L->stream;
  return 0;
}

int bk_learner_destroy(bk_learner* L) {
  delete L;
  return 0;
}

}  // extern "C"

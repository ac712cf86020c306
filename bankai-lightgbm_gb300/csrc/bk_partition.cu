// DataPartition::Split (data_partition.rs:124-174), GB300 form: a stable partition of the
// split leaf's row-index range into the left rows (kept in leaf order) followed by the right
// rows (kept in leaf order), written into the other index buffer. When the rows' order inside a
// child cannot change any result (no leaf renewal), the batched grow loop uses a single-pass
// form instead (k_part_onepass, below).
//
// The reference routes each row through SplitRule::route_bin; here every CTA evaluates that rule
// once per stored bin into a 256-entry shared route table, so routing a row is one byte read of
// the split feature's column-major bins plus one shared-memory lookup. Two kernels on a fixed grid
// (so the step can be captured in a CUDA graph while the leaf size varies): count the left rows
// of each CTA's contiguous chunk; then scatter, each CTA summing the counts of the chunks before
// its own (at most a few hundred) and ordering its rows with block-wide scans.
#include "bk_decide.cuh"
#include "bk_grow.cuh"
#include "bk_launch.cuh"

namespace bk {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;

struct PartRange {
  int64_t begin, count, r0, r1;
  int active;  // CTAs with rows: ceil(count / chunk)
  const int32_t* src;
  int32_t* dst;
  const uint8_t* col;
  // quantized path: the packed values move with the row indices; the root's are read by row
  const int16_t* pk_src;
  int16_t* pk_dst;
  bool pk_row;
};

__device__ __forceinline__ int32_t part_pk(const PartRange& R, int64_t e, int32_t row) {
  return R.pk_row ? R.pk_src[row] : R.pk_src[e];
}

// The split recorded in the job state (the search launch decided it).
__device__ __forceinline__ Decision recorded_decision(const JobState* st) {
  Decision d;
  d.stop = st->stop;
  d.leaf = st->split_leaf;
  d.inner = st->split_inner;
  d.thr = st->split_thr;
  d.begin = st->split_begin;
  d.count = st->split_count;
  d.buf = st->split_buf;
  d.depth = st->split_depth;
  d.sslot = st->split_sslot;
  d.new_leaf = st->new_leaf;
  d.pslot = st->split_pslot;
  return d;
}

__device__ __forceinline__ void part_range(const Job& J, const Params& p, const uint8_t* bins_cm, const Decision& d,
                                           PartRange* r) {
  r->begin = d.begin;
  r->count = d.count;
  const int32_t buf = d.buf;
  r->src = leaf_idx(J, buf) + r->begin;
  r->dst = leaf_idx_w(J, 1 - buf) + r->begin;
  r->col = bins_cm + (size_t)d.inner * (size_t)p.n;
  r->pk_row = d.new_leaf == 1;  // the root (one leaf when decided): no leaf-ordered copy yet
  r->pk_src = p.quant ? (r->pk_row ? J.packed : leaf_pk(J, buf) + r->begin) : nullptr;
  r->pk_dst = p.quant ? leaf_pk(J, 1 - buf) + r->begin : nullptr;
  // rows per CTA in multiples of one row per thread: a small leaf spreads over as many CTAs as
  // it fills, so each CTA's gather of the split column is short
  int64_t chunk = ceil_div64(r->count, p.part_grid);
  chunk = (chunk + kThreads - 1) / kThreads * kThreads;
  if (chunk < kThreads) chunk = kThreads;
  r->r0 = min((int64_t)blockIdx.x * chunk, r->count);
  r->r1 = min(r->r0 + chunk, r->count);
  r->active = (int)ceil_div64(r->count, chunk);
}

template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* total, T* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += u;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T w = lane < (int)(blockDim.x >> 5) ? sh[lane] : (T)0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    if (lane < (int)(blockDim.x >> 5)) sh[lane] = w;
  }
  __syncthreads();
  T warp_prefix = warp > 0 ? sh[warp - 1] : (T)0;
  *total = sh[(blockDim.x >> 5) - 1];
  T excl = warp_prefix + x - v;
  __syncthreads();
  return excl;
}

// The route of every stored bin of the chosen split (data_partition.rs:299-410), one per thread,
// from the split feature's metadata `m` (gbins, default_bin, mfb, missing, cat, offset).
// A categorical split routes by the bitset of its left bins, kept in the chosen leaf's candidate
// (data_partition.rs:264-300 and route_bin :367-377): group bin 0 (the most frequent bin's rows)
// goes left when the most frequent bin is not 0 and is in the bitset; stored bin b looks up bit
// b - 1 + offset.
__device__ __forceinline__ void build_route_of(const Job& J, const Params& p, const Decision& d, const DevFeature m,
                                               uint8_t* lut) {
  const uint32_t b = threadIdx.x;
  if (m.cat) {
    const uint32_t* bits = cand_cat_bits(J, p, d.leaf, d.inner);
    const uint32_t pos = b == 0 ? (uint32_t)m.mfb : b - 1 + (uint32_t)m.offset;
    const bool set = pos < 256u && ((__ldcg(bits + (pos >> 5)) >> (pos & 31)) & 1u) != 0u;
    lut[b] = ((int)b < m.gbins && set && (b != 0 || m.mfb > 0)) ? 1 : 0;
    return;
  }
  const uint32_t th = d.thr;
  lut[b] = (int)b < m.gbins ? route_bin(m, th & 0x7fffffffu, (th >> 31) != 0, b) : 0;
}

__device__ __forceinline__ void build_route(const Job& J, const Params& p, const Decision& d,
                                            const DevFeature* feats, uint8_t* lut) {
  build_route_of(J, p, d, feats[d.inner], lut);
}

// What build_route needs of a feature, packed in 8 bytes so a CTA can hold every feature's in
// shared memory before the split is known: x = gbins | default_bin << 16, y = mfb | missing << 16 |
// cat << 20 | offset << 21.
constexpr int kRoutePrefetch = 1024;  // features whose descriptors a partition CTA keeps

__device__ __forceinline__ uint2 route_desc(const DevFeature& m) {
  return make_uint2((uint32_t)m.gbins | ((uint32_t)m.default_bin << 16),
                    (uint32_t)m.mfb | ((uint32_t)m.missing << 16) | ((uint32_t)(m.cat != 0) << 20) |
                        ((uint32_t)m.offset << 21));
}

__device__ __forceinline__ DevFeature route_feature(uint2 q) {
  DevFeature m{};
  m.gbins = (int32_t)(q.x & 0xffffu);
  m.default_bin = (int32_t)(q.x >> 16);
  m.mfb = (int32_t)(q.y & 0xffffu);
  m.missing = (int32_t)((q.y >> 16) & 15u);
  m.cat = (int32_t)((q.y >> 20) & 1u);
  m.offset = (int32_t)((q.y >> 21) & 1u);
  return m;
}

__global__ void __launch_bounds__(kThreads) k_part_count(const JobTable jobs, Params p,
                                                         const uint8_t* __restrict__ bins_cm,
                                                         const DevFeature* __restrict__ feats) {
  __shared__ uint8_t lut[256];
  __shared__ int64_t sh[32];
  griddep_wait();
  const Job& J = jobs.job[blockIdx.z];
  if (J.st->stop) return;
  const Decision dec = recorded_decision(J.st);
  PartRange R;
  part_range(J, p, bins_cm, dec, &R);  // its loads are in flight with the route table's
  build_route(J, p, dec, feats, lut);
  __syncthreads();
  if ((int)blockIdx.x >= R.active) {  // no rows: the scatter reads only active CTAs' counts
    griddep_launch();
    return;
  }
  // per tile: every row index first, then every bin byte, so a tile costs two memory round trips
  int64_t local = 0;
  for (int64_t base = R.r0; base < R.r1; base += kThreads * kItems) {
    int32_t rows[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int64_t e = base + (int64_t)k * kThreads + threadIdx.x;
      rows[k] = e < R.r1 ? __ldg(R.src + e) : -1;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k)
      if (rows[k] >= 0) local += lut[__ldg(R.col + rows[k])];
  }
  griddep_launch();
  int64_t total;
  block_excl_scan<int64_t>(local, &total, sh);
  if (threadIdx.x == 0) J.part_cnt[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) k_part_scatter(const JobTable jobs, Params p,
                                                           const uint8_t* __restrict__ bins_cm,
                                                           const DevFeature* __restrict__ feats) {
  __shared__ uint8_t lut[256];
  __shared__ int32_t sh[32];
  griddep_wait();
  const Job& J = jobs.job[blockIdx.z];
  if (J.st->stop) return;
  __shared__ int64_t sh64[32];
  const Decision dec = recorded_decision(J.st);
  PartRange R;
  part_range(J, p, bins_cm, dec, &R);  // its loads are in flight with the route table's
  build_route(J, p, dec, feats, lut);
  __syncthreads();
  // left rows before this chunk, and in total
  int64_t before = 0, all = 0;
  const bool active = (int)blockIdx.x < R.active;
  for (int i = threadIdx.x; active && i < R.active; i += kThreads) {
    int64_t c = J.part_cnt[i];
    all += c;
    if (i < (int)blockIdx.x) before += c;
  }
  int64_t total_left = 0, running = 0;
  if (active) {
    block_excl_scan<int64_t>(all, &total_left, sh64);
    block_excl_scan<int64_t>(before, &running, sh64);
    if (blockIdx.x == 0 && threadIdx.x == 0) J.st->total_left = total_left;
  }
  for (int64_t base = R.r0; base < R.r1; base += kThreads * kItems) {
    int64_t e0 = base + (int64_t)threadIdx.x * kItems;
    int32_t rows[kItems];
    uint32_t flags = 0;
    int32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) rows[k] = e0 + k < R.r1 ? __ldg(R.src + e0 + k) : -1;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
      if (rows[k] >= 0 && lut[__ldg(R.col + rows[k])]) {
        flags |= 1u << k;
        ++cnt;
      }
    int32_t tile_total;
    int32_t pre = block_excl_scan<int32_t>(cnt, &tile_total, sh);
    int64_t left_before = running + pre;
    int32_t pkv[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) pkv[k] = (p.quant && rows[k] >= 0) ? part_pk(R, e0 + k, rows[k]) : 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      int64_t e = e0 + k;
      if (e < R.r1) {
        const int64_t slot = (flags & (1u << k)) ? left_before++ : total_left + (e - left_before);
        R.dst[slot] = rows[k];
        if (p.quant) R.pk_dst[slot] = (int16_t)pkv[k];
      }
    }
    running += tile_total;
  }
  griddep_launch();  // only the last CTA's bookkeeping is left: the next histogram may be scheduled
  // the last CTA of the launch applies the split to the leaf records (bk_grow.cuh)
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned t = atomicAdd(&J.st->part_done, 1u);
    last = t == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x < 32) post_split_body(J, p, feats);
  if (threadIdx.x == 0) J.st->part_done = 0u;
}

// Single-pass partition, for when the order of a child's rows inside its range cannot change any
// result (no leaf renewal: integer histograms, the score update and the row -> leaf map do not
// depend on it). Each 2048-row tile claims the slots of its left rows from the front of the
// range and those of its right rows from the back, one atomic each on the counter pair of this
// split's parity; inside a tile the rows keep their leaf order. No count pass and no serial tail:
// the histogram launch that follows reads the left total and applies the split's bookkeeping
// (bk_grow.cuh), and the search after it clears the counter pair for the split after next.
__global__ void __launch_bounds__(kThreads) k_part_onepass(const JobTable jobs, Params p,
                                                           const uint8_t* __restrict__ bins_cm,
                                                           const DevFeature* __restrict__ feats, int par,
                                                           int decide) {
  static_assert(kThreads == kDecideThreads, "the partition CTA runs the split decision");
  __shared__ uint8_t lut[256];
  __shared__ int64_t s_off[2];
  __shared__ Decision dec;
  __shared__ uint2 s_route[kRoutePrefetch];
  __shared__ DecideSmem ds;
  // static: every feature's route descriptor, read while the search finishes
  const bool prefetched = p.F <= kRoutePrefetch;
  if (prefetched)
    for (int f = threadIdx.x; f < p.F; f += kThreads) s_route[f] = route_desc(feats[f]);
  // the leaf arg-max over the leaves the search does not cover, while the search runs (their
  // records come from the histogram launch of this step and earlier, complete by the time the
  // search lets this launch start)
  const Job& Jpre = jobs.job[blockIdx.z];
  if (decide) decide_leaves(Jpre, p, ds);
  griddep_wait();
  // the next histogram launch may be scheduled now: its CTAs zero their shared histograms while
  // this partition runs, and wait for its completion before reading anything it writes
  griddep_launch();
  const Job& J = jobs.job[blockIdx.z];
  JobState* st = J.st;
  if (decide) {
    // every CTA decides the split from the search's records (a stopped tree included: the stop
    // flag comes with part one's loads); CTA 0 records it
    __syncthreads();
    decide_finish(J, p, feats, blockIdx.x == 0, &dec, ds);
  } else if (threadIdx.x == 0) {
    dec = recorded_decision(st);
  }
  __syncthreads();
  if (dec.stop) return;
  PartRange R;
  part_range(J, p, bins_cm, dec, &R);
  if ((int)blockIdx.x >= R.active) return;  // CTAs past the leaf's rows leave at once
  if (prefetched) build_route_of(J, p, dec, route_feature(s_route[dec.inner]), lut);
  else build_route(J, p, dec, feats, lut);
  __syncthreads();
  unsigned long long* cnt_left = reinterpret_cast<unsigned long long*>(&st->pcnt[par][0]);
  unsigned long long* cnt_right = reinterpret_cast<unsigned long long*>(&st->pcnt[par][1]);
  __shared__ int32_t s_pre[kItems][kThreads / 32];  // left rows before each (item, warp) group
  __shared__ int32_t s_tile_left;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lanes_below = (1u << lane) - 1u;
  // A tile's element j = k * kThreads + threadIdx.x (item k of this thread): every load and store
  // instruction covers 32 consecutive elements. Rows keep the tile's element order on both sides.
  for (int64_t base = R.r0; base < R.r1; base += kThreads * kItems) {
    int32_t rows[kItems];
    uint32_t flags = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int64_t e = base + k * kThreads + threadIdx.x;
      rows[k] = e < R.r1 ? __ldg(R.src + e) : -1;
    }
    int32_t pkv[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int64_t e = base + k * kThreads + threadIdx.x;
      pkv[k] = (p.quant && rows[k] >= 0) ? part_pk(R, e, rows[k]) : 0;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k)
      if (rows[k] >= 0 && lut[__ldg(R.col + rows[k])]) flags |= 1u << k;
    // left rows before each element of the tile, in element order: within the warp's 32 elements
    // of item k by ballot, across (item, warp) groups by one scan of kItems * warps counts
    int32_t in_warp[kItems];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const unsigned b = __ballot_sync(FULL, (flags >> k) & 1u);
      in_warp[k] = __popc(b & lanes_below);
      if (lane == 0) s_pre[k][warp] = __popc(b);
    }
    __syncthreads();
    if (warp == 0) {
      // kItems * warps = 64 group counts in element order (item-major), two per lane
      constexpr int kGroups = kItems * (kThreads / 32);
      static_assert(kGroups == 64, "two groups per lane");
      int32_t* flat = &s_pre[0][0];
      const int32_t c0 = flat[2 * lane], c1 = flat[2 * lane + 1];
      int32_t x = c0 + c1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
      }
      const int32_t excl = x - (c0 + c1);
      __syncwarp();
      flat[2 * lane] = excl;
      flat[2 * lane + 1] = excl + c0;
      if (lane == 31) s_tile_left = x;
    }
    __syncthreads();
    const int32_t tile_left = s_tile_left;
    const int32_t n = (int32_t)min((int64_t)kThreads * kItems, R.r1 - base);
    if (threadIdx.x == 0) {
      s_off[0] = (int64_t)atomicAdd(cnt_left, (unsigned long long)tile_left);
      s_off[1] = (int64_t)atomicAdd(cnt_right, (unsigned long long)(n - tile_left));
    }
    __syncthreads();
    // left rows fill [lo, lo + tile_left); right rows fill the tile's slots ending at count - ro
    const int64_t lo = s_off[0];
    const int64_t ro = R.count - s_off[1] - (n - tile_left);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int32_t j = k * kThreads + (int32_t)threadIdx.x;
      if (j < n) {
        const int32_t left_before = s_pre[k][warp] + in_warp[k];
        const int64_t slot = ((flags >> k) & 1u) ? lo + left_before : ro + (j - left_before);
        R.dst[slot] = rows[k];
        if (p.quant) R.pk_dst[slot] = (int16_t)pkv[k];
      }
    }
    __syncthreads();  // s_pre and s_off are rewritten by the next tile
  }
}

}  // namespace

void launch_partition(const Job* h_jobs, int num_jobs, const Params& p, const uint8_t* bins_cm,
                      const DevFeature* feats, bool stable, int par, bool decide, cudaStream_t s) {
  for_job_groups(h_jobs, num_jobs, [&](const JobTable& t, int nz) {
    dim3 grid(p.part_grid, 1, nz);
    if (stable) {
      (void)launch_kernel(k_part_count, grid, dim3(kThreads), 0, s, p.pdl, t, p, bins_cm, feats);
      (void)launch_kernel(k_part_scatter, grid, dim3(kThreads), 0, s, p.pdl, t, p, bins_cm, feats);
    } else {
      (void)launch_kernel(k_part_onepass, grid, dim3(kThreads), 0, s, p.pdl, t, p, bins_cm, feats, par,
                          decide ? 1 : 0);
    }
  });
}

}  // namespace bk

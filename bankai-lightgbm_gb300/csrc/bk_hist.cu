// ConstructHistograms for the smaller leaf (serial.rs:891-1164), GB300 form.
//
// Grid: (blocks_per_tile, T, jobs). Each CTA owns one 32-feature tile and one contiguous chunk
// of the leaf's rows. A warp takes 32 rows at a time: every lane fetches its row's run of the
// tile (32 bytes of 8-bit bins, or 16 bytes of 4-bit bins) with 128-bit loads. The CTA-private
// shared histogram keeps feature f's counters of every bin in bank f. Every lane adds its own
// row feature by feature, lane l taking feature k ^ l at step k: the 32 lanes of each shared
// atomic hit 32 different features, 32 different banks, so they never conflict and never
// collide, and no row passes through shared memory. At the end the CTA adds its non-zero bins to
// the leaf's slot in the histogram pool with global atomics (the pool slot is zeroed when the
// tree starts). Only the tile's own bins (its largest feature's group bins) are zeroed and
// flushed.
//
// A quantized CTA with few rows (at most `direct_rows`) skips the shared histogram: it stages
// each warp's 32 rows in shared memory and adds every (row, feature) to the pool slot with one
// global 64-bit atomic, lane = feature, so each atomic instruction covers 32 consecutive pool
// entries. That saves the CTA's zeroing, barrier and flush pass (with so few rows nearly every
// bin would be flushed anyway). Integer sums do not depend on the order, so both forms give the
// same slot.
//
// Quantized path: the packed int8 gradient / uint8 hessian of a row is added as one 32-bit
// value (grad << 16) + hess into a 16:16 "hot" histogram, which is folded into 32-bit
// grad/hess "cold" counters before either half can overflow, and finally into the int64
// (grad << 32) + hess pool slot. Integer sums are exact, so the result equals the reference's
// sequential i64 histogram bit for bit.
//
// Float path: gradient and hessian each go to an fp32 (hi, lo) pair: hi is updated with
// atomicAdd, which returns the previous value, and the exact rounding error of that addition
// (Knuth's TwoSum on old and addend) is added to lo. hi + lo carries the sum to about 2^-48
// relative; the pool slot receives (double)hi + (double)lo via f64 global atomics. With a
// constant hessian the hessian slot counts rows and is scaled by hessians[0] at the flush
// (serial.rs:980-988), which is exact.
//
// The last CTA of tile 0 also computes the per-leaf constants of the search that follows
// (bk_leaf.cuh) before its own rows.
#include <algorithm>
#include <mutex>

#include "bk_launch.cuh"
#include "bk_leaf.cuh"

namespace bk {

namespace {

__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  float bb = __fsub_rn(s, a);
  float e1 = __fsub_rn(a, __fsub_rn(s, bb));
  float e2 = __fsub_rn(b, bb);
  return __fadd_rn(e1, e2);
}

struct Range {
  int64_t r0, r1, count;
  const int32_t* idx;
  const int16_t* pk;  // packed values: by row for the root, else in leaf order
  int32_t slot;       // the pool slot the histogram goes to
  bool direct, pk_row;
};

// The smaller leaf's rows for this CTA: 1 with rows, 2 without rows for this CTA (r->slot set),
// 0 when the job builds no histogram in this launch (the same for every CTA of the job). With
// `post`, the previous split's single-pass partition left its bookkeeping to this launch: the
// range comes from the split's outcome (bk_grow.cuh), and the side CTA writes the bookkeeping and
// the leaf constants. Otherwise it comes from the job state and the side CTA computes the
// constants.
__device__ __forceinline__ int cta_range(const Job& J, const Params& p, int blocks_per_tile, int post, int par,
                                         Range* r) {
  const JobState* st = J.st;
  // the stop flag is loaded with the rest of the state (one round of independent loads)
  const int32_t stop = st->stop;
  int64_t begin, count;
  int32_t buf;
  if (post) {
    const SplitOutcome o = split_outcome(p, st, __ldcg(&st->pcnt[par][0]));
    if (stop) return 0;
    hist_apply_split(J, p, o);
    if (!o.go) return 0;
    begin = o.hist_begin();
    count = o.hist_count();
    buf = o.nbuf;
    r->slot = o.sslot;
    r->pk_row = false;
  } else {
    const int32_t do_search = st->do_search, slot = st->smaller_slot, leaves = st->tree_leaves;
    begin = st->hist_begin;
    count = st->hist_count;
    buf = st->hist_buf;
    if (stop) return 0;
    hist_leaf_constants(J, p);
    if (!do_search) return 0;
    r->slot = slot;
    r->pk_row = leaves == 1;  // the root: no leaf-ordered copy yet
  }
  // at least p.hist_min_rows rows per CTA (256 by default, eight warps' worth): small leaves spread
  // over as many SMs as they can fill, since a CTA's rows cost its SM's load and shared-atomic
  // pipes, not a DRAM share. Tile 0 leaves its last CTA, the side CTA, without rows (when it has
  // others), so the side work (bookkeeping, leaf constants) runs beside the rows, not before them.
  const int row_ctas = (blockIdx.y == 0 && blocks_per_tile > 1) ? blocks_per_tile - 1 : blocks_per_tile;
  int64_t chunk = ceil_div64(count, row_ctas);
  if (chunk < p.hist_min_rows) chunk = p.hist_min_rows;
  chunk = (chunk + 31) / 32 * 32;
  r->r0 = (int64_t)blockIdx.x * chunk;
  if (r->r0 >= count) return 2;
  r->r1 = min(count, r->r0 + chunk);
  r->count = count;
  r->idx = leaf_idx(J, buf) + begin;
  r->direct = (count == p.n);  // all rows in order: the index buffer is the identity
  r->pk = r->pk_row ? J.packed : (J.pk0 ? leaf_pk(J, buf) + begin : nullptr);
  return 1;
}

// The rows of a warp's round are fetched in two stages, each one round ahead of its use: the row
// index (a coalesced load of the leaf's index range, two rounds ahead) and then the row's 32-byte
// tile sector and packed value (one round ahead), so no gather waits on an index load.

struct RoundLoad {
  uint4 a, b;
  int32_t v;
};

// Positions are 32-bit: a leaf has fewer than 2^31 rows, and a lookahead position past the
// leaf's end stays below 2^32. `swap` (0 or 1) exchanges the two 16-byte halves of a 32-byte run
// as they are loaded.
__device__ __forceinline__ int32_t round_row32(const Range& R, uint32_t i, uint32_t r1) {
  if (i >= r1) return -1;
  return R.direct ? (int32_t)i : __ldg(R.idx + i);
}

__device__ __forceinline__ RoundLoad load_round_int(const uint8_t* tb, uint32_t rs, const Range& R, uint32_t i,
                                                    int32_t row, bool wide, bool half, uint32_t swap) {
  RoundLoad L;
  L.a = make_uint4(0, 0, 0, 0);
  L.b = make_uint4(0, 0, 0, 0);
  L.v = 0;
  if (row >= 0) {
    const uint4* src = reinterpret_cast<const uint4*>(tb + (size_t)(uint32_t)row * rs);
    L.a = __ldg(src + swap);
    if (!half) L.b = __ldg(src + (swap ^ 1u));
    int32_t pk = R.pk[R.pk_row ? (uint32_t)row : i];
    int32_t gi = (int32_t)(int8_t)(pk >> 8);
    int32_t hi = pk & 0xff;
    L.v = wide ? ((gi & 0xffff) | (hi << 16)) : gi * 65536 + hi;
  }
  return L;
}

// The gradient half of a 16:16 hot counter (grad * 65536 + hess, hess in [0, 65536)).
__device__ __forceinline__ int32_t hot_g(uint32_t s) { return ((int32_t)s - (int32_t)(s & 0xffffu)) >> 16; }

// Lane f's stored bin of staged row j: byte f of the row's 32-byte run, or the nibble f of its
// 16-byte run (low nibble for even f).
template <bool NIBBLE>
__device__ __forceinline__ uint32_t staged_bin(const uint8_t* sb, int j, int lane) {
  if (!NIBBLE) return sb[j * 32 + lane];
  return (sb[j * 32 + (lane >> 1)] >> ((lane & 1) << 2)) & 15u;
}

// The (grad << 32) + hess pool value of a row's packed statistics as the kernel carries them.
template <bool WIDE>
__device__ __forceinline__ unsigned long long pool_value(int32_t v) {
  const int32_t g = WIDE ? (int32_t)(int16_t)(v & 0xffff) : hot_g((uint32_t)v);
  const int32_t h = WIDE ? (v >> 16) : (v & 0xffff);
  return (unsigned long long)((int64_t)g * 4294967296LL + (int64_t)h);
}

// Shared memory of the integer kernel. Hot form: one 256-byte row per bin holding the tile's 32
// 16:16 hot counters and then its 32 cold (32-bit) gradient counters, followed by the cold
// hessian counters [bin][32]. Wide form (no hot counters): the cold gradient counters
// [bin][32], then the cold hessian ones. Feature f's counters sit in bank f either way. A CTA
// that adds straight to the pool slot (direct) uses none of them and stages its rows over the
// same bytes instead: 64 uint4 per warp, then 32 packed values per warp.
template <bool WIDE>
struct IntHist {
  static constexpr int GS = WIDE ? TILE : 2 * TILE;  // words from one bin's counters to the next
  unsigned char* base;
  int Bt;
  __device__ uint32_t* hot() const { return reinterpret_cast<uint32_t*>(base); }
  __device__ int32_t* cold_g() const { return reinterpret_cast<int32_t*>(base) + (WIDE ? 0 : TILE); }
  __device__ int32_t* cold_h() const { return reinterpret_cast<int32_t*>(base) + (size_t)Bt * GS; }
};

// Adds a row's packed value to the (bin, feature) counters of the wide form.
__device__ __forceinline__ void add_wide(const IntHist<true>& H, uint32_t bin, int32_t v, uint32_t f) {
  atomicAdd(&H.cold_g()[bin * TILE + f], (int32_t)(int16_t)(v & 0xffff));
  atomicAdd(&H.cold_h()[bin * TILE + f], v >> 16);
}

// Adds a row's packed value to the hot counter at byte offset (bin << 8) | 4 f.
__device__ __forceinline__ void add_hot(unsigned char* base, uint32_t off, int32_t v) {
  atomicAdd(reinterpret_cast<uint32_t*>(base + off), (uint32_t)v);
}

// w[i] <- w[i ^ (q & (2 TOP - 1))] (N a power of two, TOP <= N / 2): one select per word and bit.
template <int N, int TOP = N / 2>
__device__ __forceinline__ void xor_permute(uint32_t (&w)[N], uint32_t q) {
#pragma unroll
  for (int bit = TOP; bit >= 1; bit >>= 1) {
    const bool s = (q & (uint32_t)bit) != 0u;
    uint32_t t[N];
#pragma unroll
    for (int i = 0; i < N; ++i) t[i] = s ? w[i ^ bit] : w[i];
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = t[i];
  }
}

// Every lane adds its own row (its run and packed value as loaded) to the shared histogram, one
// feature per step: at step k lane l takes feature k ^ l, so the 32 lanes of each atomic hit 32
// different features — 32 different banks, whatever their bins — and no row is staged through
// shared memory or broadcast. The run's words are first permuted by the lane's high feature bits
// (a word index that varies by lane cannot be a register index) and, for 8-bit bins, the bytes of
// each word by its low bits, so step k finds its bin at a fixed position: one byte permute gives
// bin << 8, and one logic op adds the feature's offset 4 (k ^ l) to make the hot counter's byte
// offset. A 16-byte run of 8-bit bins (at most 16 features) takes feature (k ^ l) & 15 at step
// k < 16 (lanes l and l ^ 16 share a column). Features at or past nf, the tile's feature count,
// get nothing. A lane without a row carries zeros. The full 8-bit run arrives with its halves
// already exchanged for lanes 16-31 (bit 2 of the word permutation).
template <bool WIDE, bool NIBBLE>
__device__ __forceinline__ void add_own_row(const IntHist<WIDE>& H, const RoundLoad& L, uint32_t lane, bool half,
                                            uint32_t nf) {
  const int32_t v = L.v;
  if (NIBBLE) {
    // 32 features in four words, feature f at bits 4 (f & 7) of word f >> 3
    uint32_t w[4] = {L.a.x, L.a.y, L.a.z, L.a.w};
    xor_permute<4>(w, (lane >> 3) & 3u);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const uint32_t f = (uint32_t)k ^ lane;
      const uint32_t bin = (w[k >> 3] >> ((((uint32_t)k & 7u) ^ (lane & 7u)) << 2)) & 15u;
      if (f < nf) {
        if constexpr (WIDE) add_wide(H, bin, v, f);
        else add_hot(H.base, (bin << 8) | (f << 2), v);
      }
    }
    return;
  }
  // byte i of each word <- byte i ^ (lane & 3)
  const uint32_t bsel = 0x3210u ^ ((lane & 3u) * 0x1111u);
  if (half) {
    // at most 16 features in four words, feature f in byte f & 3 of word f >> 2
    uint32_t w[4] = {L.a.x, L.a.y, L.a.z, L.a.w};
    xor_permute<4>(w, (lane >> 2) & 3u);
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = __byte_perm(w[i], 0u, bsel);
    const uint32_t l4 = (lane & 15u) << 2;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t f = ((uint32_t)k ^ lane) & 15u;
      if (f < nf) {
        if constexpr (WIDE) {
          add_wide(H, __byte_perm(w[k >> 2], 0u, 0x4440u | (uint32_t)(k & 3)), v, f);
        } else {
          const uint32_t b8 = __byte_perm(w[k >> 2], 0u, 0x4404u | ((uint32_t)(k & 3) << 4));
          add_hot(H.base, b8 | (l4 ^ ((uint32_t)k << 2)), v);
        }
      }
    }
    return;
  }
  // 32 features in eight words, feature f in byte f & 3 of word f >> 2
  uint32_t w[8] = {L.a.x, L.a.y, L.a.z, L.a.w, L.b.x, L.b.y, L.b.z, L.b.w};
  xor_permute<8, 2>(w, lane >> 2);
#pragma unroll
  for (int i = 0; i < 8; ++i) w[i] = __byte_perm(w[i], 0u, bsel);
  const uint32_t l4 = lane << 2;
  if (nf >= 32u) {
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      if constexpr (WIDE) {
        add_wide(H, __byte_perm(w[k >> 2], 0u, 0x4440u | (uint32_t)(k & 3)), v, (uint32_t)k ^ lane);
      } else {
        const uint32_t b8 = __byte_perm(w[k >> 2], 0u, 0x4404u | ((uint32_t)(k & 3) << 4));
        add_hot(H.base, b8 | (l4 ^ ((uint32_t)k << 2)), v);
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const uint32_t f = (uint32_t)k ^ lane;
      if (f < nf) {
        if constexpr (WIDE) {
          add_wide(H, __byte_perm(w[k >> 2], 0u, 0x4440u | (uint32_t)(k & 3)), v, f);
        } else {
          const uint32_t b8 = __byte_perm(w[k >> 2], 0u, 0x4404u | ((uint32_t)(k & 3) << 4));
          add_hot(H.base, b8 | (l4 ^ ((uint32_t)k << 2)), v);
        }
      }
    }
  }
}

// Folds the hot counters into the cold ones and clears them. Every thread of the CTA calls it
// between barriers.
__device__ __forceinline__ void fold_hot(const IntHist<false>& H) {
  uint4* row4 = reinterpret_cast<uint4*>(H.base);   // 16 per bin: 8 hot, then 8 cold gradient
  int4* h4 = reinterpret_cast<int4*>(H.cold_h());  // 8 per bin
  for (int e = threadIdx.x; e < H.Bt * (TILE / 4); e += blockDim.x) {
    const int b = e >> 3, q = e & 7;
    uint4* hp = row4 + b * 16 + q;
    const uint4 s = *hp;
    if (s.x | s.y | s.z | s.w) {
      int4* gp = reinterpret_cast<int4*>(hp + 8);
      int4 g = *gp, h = h4[e];
      g.x += hot_g(s.x);
      g.y += hot_g(s.y);
      g.z += hot_g(s.z);
      g.w += hot_g(s.w);
      h.x += (int32_t)(s.x & 0xffffu);
      h.y += (int32_t)(s.y & 0xffffu);
      h.z += (int32_t)(s.z & 0xffffu);
      h.w += (int32_t)(s.w & 0xffffu);
      *gp = g;
      h4[e] = h;
      *hp = make_uint4(0, 0, 0, 0);
    }
  }
}

// The row loop of one integer-histogram CTA: with DIRECT every (row, feature) goes to the pool
// slot by a global atomic, otherwise to the CTA's shared histogram (the hot counters folded into
// the cold ones every `flush_rounds` rounds, before either half can overflow; the last round's
// are folded by the flush).
template <bool WIDE, bool NIBBLE, bool DIRECT>
__device__ __forceinline__ void hist_int_loop(const Params& p, const Range& R, const TileGeom& geo, const uint8_t* tb,
                                              size_t rs, int flush_rounds, unsigned long long* slot,
                                              unsigned char* smem) {
  const int tile = blockIdx.y;
  const int Bt = geo.bins;
  const bool half = geo.width == 16;  // one 16-byte run per row
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const IntHist<WIDE> H{smem, Bt};
  uint4* my_stage = reinterpret_cast<uint4*>(smem) + warp * 64;
  int32_t* my_v = reinterpret_cast<int32_t*>(reinterpret_cast<uint4*>(smem) + nwarps * 64) + warp * 32;
  const uint8_t* sb = reinterpret_cast<const uint8_t*>(my_stage);
  // lanes / features past the last feature of the last tile (padding) add nothing
  const uint32_t tile_feats = (uint32_t)min(TILE, p.F - tile * TILE);
  const bool feat_lane = (uint32_t)lane < tile_feats;
  const uint32_t r0 = (uint32_t)R.r0, r1 = (uint32_t)R.r1;
  const uint32_t per_round = (uint32_t)(TILE * nwarps);
  const uint32_t rounds = (r1 - r0 + per_round - 1u) / per_round;
  const uint32_t rs32 = (uint32_t)rs;
  // the full 8-bit path loads lanes 16-31's runs with their halves exchanged
  const uint32_t swap = (!DIRECT && !NIBBLE && !half) ? ((uint32_t)lane >> 4) & 1u : 0u;
  // software pipeline: the next round's runs and the round after's row indices are in flight
  // while this round is added up; `pos` is this lane's row position in the current round
  uint32_t pos = r0 + (uint32_t)(warp * TILE + lane);
  RoundLoad cur = load_round_int(tb, rs32, R, pos, round_row32(R, pos, r1), WIDE, half, swap);
  int32_t row_nxt = round_row32(R, pos + per_round, r1);
  int until_flush = flush_rounds;
  for (uint32_t rd = 0; rd < rounds; ++rd, pos += per_round) {
    const int32_t row_nn = round_row32(R, pos + 2u * per_round, r1);
    RoundLoad nxt = load_round_int(tb, rs32, R, pos + per_round, row_nxt, WIDE, half, swap);
    row_nxt = row_nn;
    const uint32_t base = pos - (uint32_t)lane;  // the warp's first row position of the round
    if (base < r1) {
      if (DIRECT) {
        // global atomics: the round's rows are staged so that each atomic covers one row's 32
        // features, 32 consecutive pool entries
        my_stage[lane * 2] = cur.a;
        if (!half) my_stage[lane * 2 + 1] = cur.b;
        my_v[lane] = cur.v;
        __syncwarp();
        const int jn = (int)min(32u, r1 - base);  // warp-uniform
        for (int j = 0; j < jn; ++j) {
          const uint32_t b0 = staged_bin<NIBBLE>(sb, j, lane);
          const int32_t v0 = my_v[j];
          if (feat_lane) atomicAdd(slot + b0 * TILE + lane, pool_value<WIDE>(v0));
        }
        __syncwarp();
      } else {
        add_own_row<WIDE, NIBBLE>(H, cur, (uint32_t)lane, half, tile_feats);
      }
    }
    cur = nxt;
    if constexpr (!WIDE && !DIRECT) {
      if (--until_flush == 0 && rd + 1 < rounds) {
        until_flush = flush_rounds;
        __syncthreads();
        fold_hot(H);
        __syncthreads();
      }
    }
  }
}

// The rows and flush of one integer-histogram CTA, its range known (NIBBLE: the tile holds
// 4-bit bins).
template <bool WIDE, bool NIBBLE>
__device__ __forceinline__ void hist_int_rows(const Job& J, const Params& p, const Range& R, const TileGeom& geo,
                                              const uint8_t* __restrict__ bins_rt, const uint8_t* __restrict__ bins_tm,
                                              int flush_rounds, int direct_rows, bool in_cluster, unsigned char* smem) {
  const int tile = blockIdx.y;
  const int Bt = geo.bins;
  const IntHist<WIDE> H{smem, Bt};
  unsigned long long* slot = reinterpret_cast<unsigned long long*>(J.pool) +
                             ((size_t)R.slot * p.T + tile) * (size_t)p.B * TILE;
  // uniform over the CTA; a CTA of a cluster always adds through its shared histogram
  const bool direct = !in_cluster && R.r1 - R.r0 <= (int64_t)direct_rows;
  __syncthreads();
  // the tile's run of row 0 and the row stride, in the copy that suits the leaf's density
  const bool dense = R.count * 4 >= p.n;
  const uint8_t* tb = dense ? bins_tm + geo.tm_off : bins_rt + geo.rt_off;
  const size_t rs = dense ? (size_t)tile_width(geo) : (size_t)p.rt_stride;
  if (direct) {
    hist_int_loop<WIDE, NIBBLE, true>(p, R, geo, tb, rs, flush_rounds, slot, smem);
    return;
  }
  hist_int_loop<WIDE, NIBBLE, false>(p, R, geo, tb, rs, flush_rounds, slot, smem);
  if (in_cluster) return;  // a cluster flushes its CTAs' histograms together
  __syncthreads();
  for (int e = threadIdx.x; e < Bt * TILE; e += blockDim.x) {
    const int gi = (e >> 5) * IntHist<WIDE>::GS + (e & (TILE - 1));  // (bin, feature) in the row layout
    int32_t gg = H.cold_g()[gi], hh = H.cold_h()[e];
    if (!WIDE) {
      const uint32_t s = H.hot()[gi];
      gg += hot_g(s);
      hh += (int32_t)(s & 0xffffu);
    }
    if (gg | hh) {
      int64_t pk = (int64_t)gg * 4294967296LL + (int64_t)hh;
      atomicAdd(slot + e, (unsigned long long)pk);
    }
  }
}

// The flush of a thread-block cluster of `ncta` CTAs of one feature tile: every CTA folds its
// 16:16 counters into its 32-bit ones, then (after a cluster barrier) CTA `rank` adds up its
// 1/ncta share of the tile's bins over every CTA's shared histogram through distributed shared
// memory and adds the non-zero sums to the pool slot — ncta times fewer global atomics than a
// flush per CTA. A second cluster barrier keeps every CTA's shared memory alive until the others
// have read it. Every CTA of the cluster calls it, with or without rows of its own (a CTA without
// rows contributes its zeroed histogram). Integer sums: the slot gets the same values.
template <bool WIDE>
__device__ __forceinline__ void hist_cluster_flush(const Params& p, const TileGeom& geo, unsigned long long* slot,
                                                   uint32_t ncta, unsigned char* smem) {
  const int Bt = geo.bins;
  const IntHist<WIDE> H{smem, Bt};
  const int n4 = Bt * TILE / 4;  // int4 groups of the tile's bins: a multiple of 64 (Bt a multiple of 8)
  __syncthreads();
  if constexpr (!WIDE) fold_hot(H);
  cluster_sync_all();
  const uint32_t rank = cluster_ctarank();
  const int per = n4 / (int)ncta;
  for (int e = (int)rank * per + threadIdx.x; e < ((int)rank + 1) * per; e += blockDim.x) {
    int4 g = make_int4(0, 0, 0, 0), h = make_int4(0, 0, 0, 0);
    for (uint32_t q = 0; q < ncta; ++q) {
      // int4 group e = (bin e >> 3, features 4 (e & 7) ..)
      const int4 a = ld_dsmem_v4(H.cold_g() + (e >> 3) * IntHist<WIDE>::GS + 4 * (e & 7), q);
      const int4 b = ld_dsmem_v4(H.cold_h() + 4 * e, q);
      g.x += a.x;
      g.y += a.y;
      g.z += a.z;
      g.w += a.w;
      h.x += b.x;
      h.y += b.y;
      h.z += b.z;
      h.w += b.w;
    }
    const int32_t gg[4] = {g.x, g.y, g.z, g.w}, hh[4] = {h.x, h.y, h.z, h.w};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (gg[k] | hh[k])
        atomicAdd(slot + 4 * e + k, (unsigned long long)((int64_t)gg[k] * 4294967296LL + (int64_t)hh[k]));
  }
  cluster_sync_all();
}

template <bool WIDE>
__global__ void __launch_bounds__(1024, 1)
    k_hist_int(const JobTable jobs, Params p, const uint8_t* __restrict__ bins_rt, const uint8_t* __restrict__ bins_tm,
               int blocks_per_tile, int flush_rounds, int direct_rows, int post, int par) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TileGeom geo = p.tiles[blockIdx.y];  // static: loaded while the previous kernel finishes
  // the shared histogram is zeroed while the previous kernel of the grow loop finishes
  {
    uint4* z = reinterpret_cast<uint4*>(smem);
    const int n16 = (WIDE ? 2 : 3) * geo.bins * TILE / 4;
    for (int e = threadIdx.x; e < n16; e += blockDim.x) z[e] = make_uint4(0, 0, 0, 0);
  }
  griddep_wait();
  // the search may be scheduled now: its CTAs read their static data while this launch runs, and
  // wait for its completion before reading anything it writes
  griddep_launch();
  const Job& J = jobs.job[blockIdx.z];
  Range R;
  // a cluster's CTAs belong to one job and tile, so code 0 is the same for all of them; every
  // other CTA of a cluster reaches both cluster barriers of the flush
  const uint32_t ncta = cluster_nctarank();
  const int rc = cta_range(J, p, blocks_per_tile, post, par, &R);
  if (rc == 0 || (rc == 2 && ncta == 1)) return;
  if (rc == 1) {
    if (geo.nibble)
      hist_int_rows<WIDE, true>(J, p, R, geo, bins_rt, bins_tm, flush_rounds, direct_rows, ncta > 1, smem);
    else
      hist_int_rows<WIDE, false>(J, p, R, geo, bins_rt, bins_tm, flush_rounds, direct_rows, ncta > 1, smem);
  }
  if (ncta > 1) {
    unsigned long long* slot = reinterpret_cast<unsigned long long*>(J.pool) +
                               ((size_t)R.slot * p.T + blockIdx.y) * (size_t)p.B * TILE;
    hist_cluster_flush<WIDE>(p, geo, slot, ncta, smem);
  }
}

// Adds one row's gradient (and hessian) to the fp32 (hi, lo) pairs of bin `e`: hi takes the
// value by atomicAdd, which returns the previous sum, and lo the exact rounding error of that
// addition (TwoSum); with a constant hessian the hessian slot counts rows.
template <bool CONST_HESS>
__device__ __forceinline__ void add_float(float* ghi, float* glo, float* hhi, float* hlo, uint32_t e, float2 v) {
  const float old = atomicAdd(&ghi[e], v.x);
  const float err = two_sum_err(old, v.x, __fadd_rn(old, v.x));
  if (err != 0.f) atomicAdd(&glo[e], err);
  if (CONST_HESS) {
    atomicAdd(reinterpret_cast<uint32_t*>(hhi) + e, 1u);
  } else {
    const float oh = atomicAdd(&hhi[e], v.y);
    const float eh = two_sum_err(oh, v.y, __fadd_rn(oh, v.y));
    if (eh != 0.f) atomicAdd(&hlo[e], eh);
  }
}

// The float kernel's form of add_own_row: every lane with a row adds it, feature k ^ lane at
// step k (32 different banks per atomic), from its run permuted once per row so that each step's
// bin sits at a fixed position. The full 8-bit run arrives with its halves already exchanged for
// lanes 16-31.
template <bool CONST_HESS, bool NIBBLE>
__device__ __forceinline__ void add_own_row_float(float* ghi, float* glo, float* hhi, float* hlo, const uint4& a,
                                                  const uint4& b, float2 v, uint32_t lane, bool half, uint32_t nf) {
  if (NIBBLE) {
    uint32_t w[4] = {a.x, a.y, a.z, a.w};
    xor_permute<4>(w, (lane >> 3) & 3u);
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const uint32_t f = (uint32_t)k ^ lane;
      const uint32_t bin = (w[k >> 3] >> ((((uint32_t)k & 7u) ^ (lane & 7u)) << 2)) & 15u;
      if (f < nf) add_float<CONST_HESS>(ghi, glo, hhi, hlo, bin * TILE + f, v);
    }
    return;
  }
  const uint32_t bsel = 0x3210u ^ ((lane & 3u) * 0x1111u);  // byte i of each word <- byte i ^ (lane & 3)
  if (half) {
    uint32_t w[4] = {a.x, a.y, a.z, a.w};
    xor_permute<4>(w, (lane >> 2) & 3u);
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = __byte_perm(w[i], 0u, bsel);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t f = ((uint32_t)k ^ lane) & 15u;
      const uint32_t bin = __byte_perm(w[k >> 2], 0u, 0x4440u | (uint32_t)(k & 3));
      if (f < nf) add_float<CONST_HESS>(ghi, glo, hhi, hlo, bin * TILE + f, v);
    }
    return;
  }
  uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  xor_permute<8, 2>(w, lane >> 2);
#pragma unroll
  for (int i = 0; i < 8; ++i) w[i] = __byte_perm(w[i], 0u, bsel);
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const uint32_t f = (uint32_t)k ^ lane;
    const uint32_t bin = __byte_perm(w[k >> 2], 0u, 0x4440u | (uint32_t)(k & 3));
    if (f < nf) add_float<CONST_HESS>(ghi, glo, hhi, hlo, bin * TILE + f, v);
  }
}

// The rows and flush of one float-histogram CTA, its range known (NIBBLE: the tile holds 4-bit
// bins).
template <bool CONST_HESS, bool NIBBLE>
__device__ __forceinline__ void hist_float_rows(const Job& J, const Params& p, const Range& R, const TileGeom& geo,
                                                const uint8_t* __restrict__ bins_rt,
                                                const uint8_t* __restrict__ bins_tm, unsigned char* smem) {
  const int tile = blockIdx.y;
  const int B = geo.bins;
  const bool half = geo.width == 16;  // one 16-byte run per row
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  float* ghi = reinterpret_cast<float*>(smem);
  float* glo = ghi + B * TILE;
  float* hhi = glo + B * TILE;  // CONST_HESS: uint32 row counts
  float* hlo = hhi + B * TILE;  // unused with CONST_HESS
  uint32_t* hcnt = reinterpret_cast<uint32_t*>(hhi);
  __syncthreads();
  // the tile's run of row 0 and the row stride, in the copy that suits the leaf's density
  const bool dense = R.count * 4 >= p.n;
  const uint8_t* tb = dense ? bins_tm + geo.tm_off : bins_rt + geo.rt_off;
  const uint32_t rs = dense ? (uint32_t)tile_width(geo) : (uint32_t)p.rt_stride;
  const uint32_t tile_feats = (uint32_t)min(TILE, p.F - tile * TILE);
  const float* G = J.g;
  const float* H = J.h;
  const uint32_t r0 = (uint32_t)R.r0, r1 = (uint32_t)R.r1;
  const uint32_t per_round = (uint32_t)(TILE * nwarps);
  // the full 8-bit path loads lanes 16-31's runs with their halves exchanged
  const uint32_t swap = (!NIBBLE && !half) ? ((uint32_t)lane >> 4) & 1u : 0u;
  // the same two-stage software pipeline as the integer kernel
  auto load = [&](int32_t row, uint4& a, uint4& b, float2& v) {
    a = make_uint4(0, 0, 0, 0);
    b = make_uint4(0, 0, 0, 0);
    v = make_float2(0.f, 0.f);
    if (row >= 0) {
      const uint4* src = reinterpret_cast<const uint4*>(tb + (size_t)(uint32_t)row * rs);
      a = __ldg(src + swap);
      if (!half) b = __ldg(src + (swap ^ 1u));
      v.x = G[row];
      if (!CONST_HESS) v.y = H[row];
    }
  };
  uint32_t pos = r0 + (uint32_t)(warp * TILE + lane);
  uint4 ca, cb;
  float2 cv;
  load(round_row32(R, pos, r1), ca, cb, cv);
  int32_t row_nxt = round_row32(R, pos + per_round, r1);
  for (; pos - (uint32_t)lane < r1; pos += per_round) {
    const int32_t row_nn = round_row32(R, pos + 2u * per_round, r1);
    uint4 na, nb;
    float2 nv;
    load(row_nxt, na, nb, nv);
    row_nxt = row_nn;
    if (pos < r1) add_own_row_float<CONST_HESS, NIBBLE>(ghi, glo, hhi, hlo, ca, cb, cv, (uint32_t)lane, half, tile_feats);
    ca = na;
    cb = nb;
    cv = nv;
  }
  __syncthreads();
  double2* slot = reinterpret_cast<double2*>(J.pool) + ((size_t)R.slot * p.T + tile) * (size_t)p.B * TILE;
  const double h0 = CONST_HESS ? (double)H[0] : 0.0;
  for (int e = threadIdx.x; e < B * TILE; e += blockDim.x) {
    double gs = (double)ghi[e] + (double)glo[e];
    double hs = CONST_HESS ? (double)hcnt[e] * h0 : (double)hhi[e] + (double)hlo[e];
    bool touched = CONST_HESS ? hcnt[e] != 0u : (ghi[e] != 0.f || glo[e] != 0.f || hhi[e] != 0.f || hlo[e] != 0.f);
    if (touched) {
      atomicAdd(&slot[e].x, gs);
      atomicAdd(&slot[e].y, hs);
    }
  }
}

template <bool CONST_HESS>
__global__ void __launch_bounds__(1024, 1)
    k_hist_float(const JobTable jobs, Params p, const uint8_t* __restrict__ bins_rt, const uint8_t* __restrict__ bins_tm,
                 int blocks_per_tile, int post, int par) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TileGeom geo = p.tiles[blockIdx.y];  // static: loaded while the previous kernel finishes
  {
    uint4* z = reinterpret_cast<uint4*>(smem);
    const int n16 = (CONST_HESS ? 3 : 4) * geo.bins * TILE / 4;
    for (int e = threadIdx.x; e < n16; e += blockDim.x) z[e] = make_uint4(0, 0, 0, 0);
  }
  griddep_wait();
  // the search may be scheduled now: its CTAs read their static data while this launch runs, and
  // wait for its completion before reading anything it writes
  griddep_launch();
  const Job& J = jobs.job[blockIdx.z];
  Range R;
  if (cta_range(J, p, blocks_per_tile, post, par, &R) != 1) return;
  if (geo.nibble)
    hist_float_rows<CONST_HESS, true>(J, p, R, geo, bins_rt, bins_tm, smem);
  else
    hist_float_rows<CONST_HESS, false>(J, p, R, geo, bins_rt, bins_tm, smem);
}

}  // namespace

size_t hist_smem_bytes(const Params& p, int threads, bool quant, bool wide) {
  size_t warps = (size_t)threads / 32;
  size_t stage = warps * 64 * sizeof(uint4);
  size_t bins = (size_t)p.B * TILE;
  // the integer kernel's direct CTAs stage their rows over the (unused) shared histogram
  if (quant) return std::max((wide ? 0 : bins * 4) + bins * 8, stage + warps * 32 * 4);
  if (p.const_hess) return bins * 12;
  return bins * 16;
}

void launch_hist(const Job* h_jobs, int num_jobs, const Params& p, const uint8_t* bins_rt, const uint8_t* bins_tm,
                 const HistLaunch& hl, int post, int par, cudaStream_t s) {
  for_job_groups(h_jobs, num_jobs, [&](const JobTable& t, int nz) {
    dim3 grid(hl.blocks_per_tile, p.T, nz);
    if (p.quant) {
      if (hl.flush_rounds > 0)
        (void)launch_kernel_cluster(k_hist_int<false>, grid, dim3(hl.threads), hl.smem, s, p.pdl, hl.cluster, t, p,
                                    bins_rt, bins_tm, hl.blocks_per_tile, hl.flush_rounds, hl.direct_rows, post, par);
      else
        (void)launch_kernel_cluster(k_hist_int<true>, grid, dim3(hl.threads), hl.smem, s, p.pdl, hl.cluster, t, p,
                                    bins_rt, bins_tm, hl.blocks_per_tile, 1, hl.direct_rows, post, par);
    } else if (p.const_hess) {
      (void)launch_kernel(k_hist_float<true>, grid, dim3(hl.threads), hl.smem, s, p.pdl, t, p, bins_rt, bins_tm,
                          hl.blocks_per_tile, post, par);
    } else {
      (void)launch_kernel(k_hist_float<false>, grid, dim3(hl.threads), hl.smem, s, p.pdl, t, p, bins_rt, bins_tm,
                          hl.blocks_per_tile, post, par);
    }
  });
}

cudaError_t hist_set_smem_attrs(size_t smem) {
  // The attribute belongs to the kernel on the current device: remember the largest value set on
  // each device and only ever raise it, so learners created earlier with larger tiles keep working.
  constexpr int kMaxDevices = 64;
  static std::mutex m;
  static size_t current[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(m);
  if (smem <= current[dev]) return cudaSuccess;
  int v = (int)smem;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hist_int<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hist_int<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hist_float<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_hist_float<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess) current[dev] = smem;
  return e;
}

}  // namespace bk

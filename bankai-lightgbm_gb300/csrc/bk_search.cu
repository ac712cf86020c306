// FindBestSplitsFromHistograms (serial.rs:1322-1566, int: :1212-1300) and the grow-loop
// bookkeeping kernels (serial.rs:578-628, :779-825, :1685-1876), GB300 form.
//
// k_search: one 256-thread CTA per (leaf side, feature), thread t owning local bin t (a feature
// slice holds at most 255 bins). The CTA fixes the smaller leaf's most-frequent bin (FixHistogram,
// serial.rs:2205-2238), derives the larger leaf's slice as parent minus the fixed smaller slice in
// place (serial.rs:1407-1437, :1218-1242), and evaluates both directional threshold scans of the
// reference (FindBestThresholdSequentially[Int], feature_histogram.rs:363-663 / 839-1142) at once,
// thread t holding the reverse scan's position t and the forward scan's position t. The sequential
// scan's `break` (the first threshold whose other side falls under min_data / min_hessian ends the
// scan) becomes "the first such position in scan order and everything after it is excluded";
// `current_gain > best_gain` becomes an arg-max with ties going to the earliest position in scan
// order. Every reduction is a warp reduction plus one barrier.
//
// The quantized path scans the packed (grad << 32) + hess sums with one block prefix scan; the
// reverse scan's sums are the total minus the prefix, exact in integers, so its candidates are
// bit-identical to the reference's. The float path scans f64 prefix and suffix sums (associated
// differently from the sequential scan, about 1e-16 relative).
//
// f64 is slow on this part, so it stays off the common path: the leaf constants the scans share
// come precomputed from the histogram launch (bk_leaf.cuh), plain gains are filtered in fp32 with
// a rigorous error bound, and every comparison of the fold and the arg-max runs on integer keys.
// The last CTA of k_search folds the per-feature candidates of each searched leaf in feature order
// with `better_than`, takes the arg-max leaf (split_info.rs:88-96), stops the tree when its gain is
// <= 0, and builds the route table of the chosen split (data_partition.rs:299-410). The post-split
// bookkeeping (bk_grow.cuh) runs in the last CTA of the partition scatter.
#include <math_constants.h>

#include <type_traits>

#include "bk_decide.cuh"
#include "bk_grow.cuh"
#include "bk_launch.cuh"
#include "bk_leaf.cuh"
#include "bk_math.cuh"

namespace bk {

namespace {

constexpr int kSearchThreads = kDecideThreads;  // one thread per local bin
constexpr int kSearchWarps = kSearchThreads / 32;

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Inclusive scan towards lower lanes: lane l gets the sum over lanes l .. 31.
template <typename T>
__device__ __forceinline__ T warp_incl_scan_down(T v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T u = __shfl_down_sync(FULL, v, o);
    if (lane + o < 32) v += u;
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}


__device__ __forceinline__ int64_t unpack_g(int64_t pk) { return pk >> 32; }
__device__ __forceinline__ int64_t unpack_h(int64_t pk) { return pk & 0xffffffffLL; }

// Order-preserving integer keys of non-NaN floats and doubles (negative zero counts as zero),
// computed with integer operations only.
__device__ __forceinline__ int32_t float_key(float x) {
  int32_t b = __float_as_int(x);
  if (b == (int32_t)0x80000000) b = 0;
  return b ^ ((b >> 31) & 0x7fffffff);
}
// ---- fp32 prefilter of the plain split gain (no L1 / max_delta_step / path_smooth) ----
// The reference evaluates gl^2/(hl+l2) + gr^2/(hr+l2) in f64 for every threshold. Each candidate is
// first evaluated in fp32 together with a rigorous bound E on |fp32 - f64| (u = 2^-24): the
// numerators' conversions and scaling (3u), the denominators' (4u, plus kEpsilon, below 0.02u for
// denominators >= 1e-6), the square (u), the division (__fdividef: at most 2 ulp = 4u for divisors
// in [2^-126, 2^126]) and the sum (u) add up to at most 16.1u relative to the non-negative result;
// the fp32 bound computations round once more. E uses 24u. The largest gain G* of a direction is
// at least the best certified lower bound M over its valid thresholds, so only the thresholds
// whose upper bound reaches M (and exceeds min_gain_shift) can hold it, and the direction is
// splittable exactly when G* passes min_gain_shift. Those few thresholds (and any whose fp32
// evaluation is uncertain) are evaluated in f64, so the chosen split, its gain and the splittable
// flag are exactly the reference's. A threshold whose accumulated side gained nothing since its
// predecessor in scan order (an empty bin between them) has that predecessor's gain exactly and
// comes after it, so it is never queued.
constexpr float kPrefilterRel = 24.0f * 5.9604645e-08f;

struct Approx {
  float g, e;
  bool uncertain;
};

__device__ __forceinline__ Approx approx_from(float xl, float yl, float xr, float yr) {
  Approx a;
  float tl = __fdividef(__fmul_rn(xl, xl), yl);
  float tr = __fdividef(__fmul_rn(xr, xr), yr);
  a.g = __fadd_rn(tl, tr);
  a.e = __fadd_rn(__fmul_rn(kPrefilterRel, a.g), 1e-30f);
  // non-finite values, denominators outside [1e-6, 1e30] (where the reference's +kEpsilon matters
  // or the fast division leaves its accuracy range) and huge results go to f64
  a.uncertain = !(yl >= 1e-6f) || !(yr >= 1e-6f) || !(yl <= 1e30f) || !(yr <= 1e30f) || !(a.g < 1e30f) ||
                isnan(a.g);
  return a;
}

// The quantized sums fit in 32 bits (signed gradients, unsigned hessians), so the conversions are
// single 32-bit ones.
__device__ __forceinline__ Approx approx_int(int64_t lg, int64_t lh, int64_t tg, int64_t th, float gsf, float hsf,
                                             float l2f) {
  const int64_t rg = tg - lg, rh = th - lh;
  return approx_from(__fmul_rn((float)(int32_t)lg, gsf), __fadd_rn(__fmul_rn((float)(uint32_t)lh, hsf), l2f),
                     __fmul_rn((float)(int32_t)rg, gsf), __fadd_rn(__fmul_rn((float)(uint32_t)rh, hsf), l2f));
}

// GetSplitGains of one integer threshold (feature_histogram.rs:878-925: the hessians get
// kEpsilon added, counts are round_int(hess * cnt_factor)).
__device__ __forceinline__ double int_split_gain(const Params& p, int64_t lg, int64_t lh, int64_t tg, int64_t th,
                                                 double gs, double hs, double cnt_factor, double parent, bool plain) {
  // the sums fit in 32 bits (signed gradients, unsigned hessians): 32-bit conversions, exact
  const int64_t rg = tg - lg, rh = th - lh;
  const double slh = (double)(uint32_t)lh * hs, srh = (double)(uint32_t)rh * hs;
  const int32_t lc = plain ? 0 : round_int((double)(uint32_t)lh * cnt_factor);
  const int32_t rc = plain ? 0 : round_int((double)(uint32_t)rh * cnt_factor);
  return split_gains(p, (double)(int32_t)lg * gs, slh + BK_EPS, (double)(int32_t)rg * gs, srh + BK_EPS, lc, rc,
                     parent);
}

// What one search CTA needs of the job state, loaded in one round of independent loads: the
// searched leaf's constants and sums (computed by the histogram launch), the smaller leaf's sums
// (for FixHistogram), and the pool slots of the smaller and larger leaf.
struct SearchIn {
  LeafConst C;
  LeafSum S0;
  int32_t sslot, lslot;
  // the integer search's two pool entries of this thread (IntPool), loaded from the slots known
  // before the wait; valid when those slots are the state's
  int64_t sv, lv;
  bool pre;
};

// The pool entries thread t of an integer search scans: the smaller leaf's bin t + 1 of feature
// f (none at the most-frequent bin, which the fix rewrites) and, on side 1, the larger leaf's.
struct IntPool {
  int64_t sv, lv;
};
__device__ __forceinline__ IntPool int_pool(const Job& J, const Params& p, const DevFeature& m, int side, int32_t f,
                                            int32_t sslot, int32_t lslot) {
  const int t = threadIdx.x;
  const size_t slot_stride = (size_t)p.T * p.B * TILE;
  const size_t feat_off = (size_t)(f / TILE) * p.B * TILE + (f % TILE) + (size_t)(t + 1) * TILE;
  const int64_t* pool = reinterpret_cast<const int64_t*>(J.pool);
  const bool fix = m.mfb > 0;
  const bool in = t < m.len;
  IntPool r;
  r.sv = (in && !(fix && t == m.mfb)) ? pool[(size_t)sslot * slot_stride + feat_off] : 0;
  r.lv = (side && in) ? pool[(size_t)lslot * slot_stride + feat_off] : 0;
  return r;
}

__device__ void cand_reset(Cand* c, int32_t real, int32_t inner) {
  c->gain = -CUDART_INF;
  c->left_output = c->right_output = 0.0;
  c->lsg = c->lsh = c->rsg = c->rsh = 0.0;
  c->lint = c->rint = 0;
  c->feature = real;
  c->inner = inner;
  c->threshold = 0;
  c->left_count = c->right_count = 0;
  c->default_left = 1;
  c->splittable = 0;
  c->categorical = 0;
}

// Direction geometry of FindBestThreshold[Int] (feature_histogram.rs:219-357, :673-830): direction
// 0 is the reverse scan (right side accumulates, default left, positions t = tf_r down to 1 - off),
// direction 1 the forward scan (left side accumulates, positions t = -1 or 0 up to t_end).
struct ScanGeom {
  bool two, skip, fwd_rest;
  int off, tf_r, t_end;
};

__device__ __forceinline__ ScanGeom scan_geom(const DevFeature& m) {
  ScanGeom G;
  G.two = m.num_bin > 2 && m.missing != 0;
  G.skip = G.two && m.missing == 1;
  const bool na = G.two && m.missing == 2;
  G.off = m.offset;
  G.tf_r = m.num_bin - 1 - G.off - (na ? 1 : 0);
  G.t_end = m.num_bin - 2 - G.off;
  // with NaN missing and the most-frequent bin 0, the forward scan's left side starts as
  // everything outside the slice, at position t = -1 (held by the last thread)
  G.fwd_rest = na && G.off == 1;
  return G;
}

// Scan order: the reverse scan visits higher bins first, the forward scan lower bins first.
__device__ __forceinline__ bool earlier(int d, int ta, int tb) { return d == 0 ? ta > tb : ta < tb; }

// The best position of one direction within a warp (and, combined, within the CTA).
// Everything a candidate threshold contributes to its SplitInfo: the gain, the left / right sums,
// counts and outputs.
struct Eval {
  double gain, lsg, lsh, rsg, rsh, lo, ro;
  int32_t lc, rc;
  int64_t lint, rint;
};

struct DirBest {
  long long key;  // dkey of the gain; kNoKey when no position qualified
  int64_t a, b;   // int: left (grad, hess) sums; float: bit patterns of the accumulated (grad, hess)
  int32_t t, c;   // position; float: accumulated count
  Eval ev;        // ev.gain: -inf when none
};


// The chosen threshold's SplitInfo: lane 0 evaluates the left side, lane 1 the right side, in one
// instruction stream (FindBestThresholdInt's output assembly, feature_histogram.rs:700-830: 32-bit
// conversions of the packed sums, exact since they fit in 32 bits).
__device__ __forceinline__ Eval eval_int(const Params& p, int64_t lg, int64_t lh, int64_t tg, int64_t th, double gs,
                                         double hs, double cnt_factor, double parent, double gain, int lane) {
  const int64_t rg = tg - lg, rh = th - lh;
  const int64_t sg = lane == 0 ? lg : rg, sh = lane == 0 ? lh : rh;
  const double dg = (double)(int32_t)sg * gs, dh = (double)(uint32_t)sh * hs;
  const int32_t n = round_int((double)(uint32_t)sh * cnt_factor);
  const double out = lane < 2 ? split_output(p, dg, dh, n, parent) : 0.0;
  Eval v;
  v.gain = gain;
  v.lsg = dg;
  v.lsh = dh;
  v.lc = n;
  v.lo = out;
  v.rsg = __shfl_sync(FULL, dg, 1);
  v.rsh = __shfl_sync(FULL, dh, 1);
  v.rc = __shfl_sync(FULL, n, 1);
  v.ro = __shfl_sync(FULL, out, 1);
  v.lint = (int64_t)(((uint64_t)lg << 32) | ((uint64_t)lh & 0xffffffffull));
  v.rint = (int64_t)(((uint64_t)rg << 32) | ((uint64_t)rh & 0xffffffffull));
  return v;
}

// FindBestThreshold's output assembly (feature_histogram.rs:240-357): (ag, ah, c) is the
// accumulated side of direction d (0: right, 1: left); the right side of the outputs derives from
// the left sums. Lane 0 evaluates the left output, lane 1 the right one.
__device__ __forceinline__ Eval eval_float(const Params& p, int d, double ag, double ah, int32_t c, double sum_g,
                                           double sum_h, int32_t num_data, double parent, double gain, int lane) {
  const double slg = d == 0 ? sum_g - ag : ag, slh = d == 0 ? sum_h - ah : ah;
  const int32_t lc = d == 0 ? num_data - c : c;
  const double sg = lane == 0 ? slg : sum_g - slg, sh = lane == 0 ? slh : sum_h - slh;
  const int32_t n = lane == 0 ? lc : num_data - lc;
  const double out = lane < 2 ? split_output(p, sg, sh, n, parent) : 0.0;
  Eval v;
  v.gain = gain;
  v.lsg = slg;
  v.lsh = slh - BK_EPS;
  v.lc = lc;
  v.lo = out;
  v.rsg = sum_g - slg;
  v.rsh = (sum_h - slh) - BK_EPS;
  v.rc = num_data - lc;
  v.ro = __shfl_sync(FULL, out, 1);
  v.lint = v.rint = 0;
  return v;
}

// One quarter of a queued position's evaluation, as one lane computes it (plain gains: no L1,
// max_delta_step or path_smooth). Role 0 / 1: the left / right leaf gain (simd.rs:6-8,
// feature_histogram.rs:148-176: left + right = the split gain, in that order); role 2 / 3: the
// left / right output (feature_histogram.rs:79-104) with the side's SplitInfo sums and count
// (feature_histogram.rs:240-357, :700-830). Both are one division, num / (den + lambda_l2), so all
// four lanes run the same instructions: gain = g^2 / (h + l2), output = -g / (h + l2).
struct SidePart {
  double val;     // the leaf gain (roles 0, 1) or the output (roles 2, 3)
  double sg, sh;  // the side's sums as the SplitInfo stores them (roles 2, 3)
  int32_t n;      // the side's count (roles 2, 3)
};

// Role `role` of an integer threshold with left sums (lg, lh): the hessian gets kEpsilon added for
// the gain (feature_histogram.rs:878-925), the output and the SplitInfo use the plain sums, the
// counts are round_int(hess * cnt_factor) — exactly as int_split_gain and eval_int compute them.
__device__ __forceinline__ SidePart int_side(const Params& p, int64_t lg, int64_t lh, int64_t tg, int64_t th,
                                             double gs, double hs, double cnt_factor, int role) {
  const bool right = (role & 1) != 0, gain = role < 2;
  const int64_t sg = right ? tg - lg : lg, sh = right ? th - lh : lh;
  const double dg = (double)(int32_t)sg * gs, dh = (double)(uint32_t)sh * hs;
  SidePart r;
  r.n = round_int((double)(uint32_t)sh * cnt_factor);
  const double sq = dg * dg;
  const double he = dh + BK_EPS;
  const double num = gain ? sq : -dg;
  const double den = (gain ? he : dh) + p.l2;
  r.val = num / den;
  r.sg = dg;
  r.sh = dh;
  return r;
}

// Role `role` of a float threshold of direction d with accumulated sums (ag, ah, c): the gain
// takes the sums split_gains gets (the reverse scan's right side is the accumulated one), the
// output and the SplitInfo the right side from the left sums, as eval_float computes them.
__device__ __forceinline__ SidePart float_side(const Params& p, int d, double ag, double ah, int32_t c, double sum_g,
                                               double sum_h, int32_t num_data, int role) {
  const bool right = (role & 1) != 0, gain = role < 2;
  const double slg = d == 0 ? sum_g - ag : ag, slh = d == 0 ? sum_h - ah : ah;
  const int32_t lc = d == 0 ? num_data - c : c;
  // the gain's sums: the accumulated side as accumulated, the other as total minus it
  const double gg = !right ? slg : (d == 0 ? ag : sum_g - ag);
  const double gh = !right ? slh : (d == 0 ? ah : sum_h - ah);
  // the SplitInfo's sums: the right side from the left sums
  const double og = !right ? slg : sum_g - slg, oh = !right ? slh : sum_h - slh;
  SidePart r;
  r.n = !right ? lc : num_data - lc;
  const double sq = gg * gg;
  const double num = gain ? sq : -og;
  const double den = (gain ? gh : oh) + p.l2;
  r.val = num / den;
  r.sg = og;
  r.sh = oh - BK_EPS;
  return r;
}

// One direction's stop / prefilter summary of a warp (published before one barrier).
struct WarpFilt {
  int32_t lb;      // the warp's first `break` position in scan order (kNoneLo / kNoneHi: none)
  int32_t mb, ma;  // best certified fp32 lower-bound key of positions before lb / of all positions
};

constexpr int kNoneLo = -0x7fffffff, kNoneHi = 0x7fffffff;

// A position queued for its f64 gain (PLAIN gains): evaluated by warp 0.
struct QEnt {
  int64_t a, b;  // int: left (grad, hess) sums; float: bit patterns of the accumulated (grad, hess)
  int32_t c;     // float: accumulated count
  int16_t t, d;  // position, direction
};

// The shared memory of a numerical search CTA of NW warps (32 * NW threads, one per local bin).
template <int NW>
struct SearchSmemT {
  QEnt q[2][32 * NW];  // per direction: every position at most once
  int32_t qn[2];
  DirBest pres[2][4];  // per direction and batch lane (below): the arg-max of its batches
  int32_t psplit[2][4];
  int64_t wi[2][NW];
  double wd[10][NW];
  int32_t wc[3][NW];
  WarpFilt wf[2][NW];
  WarpFilt xf;  // the forward scan's position -1 (last thread)
  int32_t spl[2][NW];
  DirBest wb[2][NW];
};
using SearchSmem = SearchSmemT<kSearchWarps>;

// This warp's arg-max of direction d (highest key, then the earliest position in scan order) into w.
__device__ __forceinline__ void warp_best(int d, bool elig, double gain, int t, int64_t a, int64_t b, int32_t c,
                                          int lane, DirBest* w) {
  const long long key = elig ? dkey(gain) : kNoKey;
  const long long km = warp_max64(key);
  if (km == kNoKey) {
    if (lane == 0) {
      w->key = kNoKey;
      w->ev.gain = -CUDART_INF;
      w->t = 0;
    }
    return;
  }
  const bool at = elig && key == km;
  const int tb = d == 0 ? __reduce_max_sync(FULL, at ? t : kNoneLo) : __reduce_min_sync(FULL, at ? t : kNoneHi);
  if (at && t == tb) {
    w->key = km;
    w->a = a;
    w->b = b;
    w->t = t;
    w->c = c;
    w->ev.gain = gain;
  }
}

// Warp 0 after the barrier: the CTA's best of each direction (lane 0: direction 0, lane 8:
// direction 1), broadcast to every lane of the warp.
template <int NW>
__device__ __forceinline__ void combine_best(const SearchSmemT<NW>& sm, int lane, DirBest (&r)[2], int (&split)[2]) {
  const int d = (lane >> 3) & 1;
  long long key = kNoKey;
  double gain = -CUDART_INF;
  int64_t a = 0, b = 0;
  int32_t t = 0, c = 0;
  int sp = 0;
  if (lane < 16 && (lane & 7) < NW) {
    const DirBest& e = sm.wb[d][lane & 7];
    key = e.key;
    if (key != kNoKey) {
      gain = e.ev.gain;
      a = e.a;
      b = e.b;
      t = e.t;
      c = e.c;
    }
    sp = sm.spl[d][lane & 7];
  }
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const long long xk = __shfl_xor_sync(FULL, key, o);
    const double xg = __shfl_xor_sync(FULL, gain, o);
    const int64_t xa = __shfl_xor_sync(FULL, a, o), xb = __shfl_xor_sync(FULL, b, o);
    const int32_t xt = __shfl_xor_sync(FULL, t, o), xc = __shfl_xor_sync(FULL, c, o);
    sp |= __shfl_xor_sync(FULL, sp, o);
    if (xk > key || (xk == key && xk != kNoKey && earlier(d, xt, t))) {
      key = xk;
      gain = xg;
      a = xa;
      b = xb;
      t = xt;
      c = xc;
    }
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int src = 8 * k;
    r[k].key = __shfl_sync(FULL, key, src);
    r[k].ev.gain = __shfl_sync(FULL, gain, src);
    r[k].a = __shfl_sync(FULL, a, src);
    r[k].b = __shfl_sync(FULL, b, src);
    r[k].t = __shfl_sync(FULL, t, src);
    r[k].c = __shfl_sync(FULL, c, src);
    split[k] |= __shfl_sync(FULL, sp, src);
  }
}

// The fp32 view of one position: certified lower-bound key lo, upper-bound key up, and whether it
// may pass min_gain_shift (mp).
struct Filt {
  bool mp, unc;
  int32_t lo, up;
};

__device__ __forceinline__ Filt filt_of(bool cand, const Approx& a, const LeafConst& C) {
  Filt f;
  f.unc = a.uncertain;
  f.mp = cand && (a.uncertain || __fadd_rn(a.g, a.e) > C.mgs_dn);
  f.lo = (cand && !a.uncertain) ? float_key(__fsub_rn(a.g, a.e)) : float_key(-CUDART_INF_F);
  f.up = a.uncertain ? 0 : float_key(__fadd_rn(a.g, a.e));
  return f;
}

// Before the barrier: the warp's summary of direction d for positions `pos` (thread order = t).
template <bool PLAIN, int NW>
__device__ __forceinline__ void publish_dir(SearchSmemT<NW>& sm, int d, bool brk, int pos, const Filt& f, int lane,
                                            int warp) {
  const int lb = d == 0 ? __reduce_max_sync(FULL, brk ? pos : kNoneLo) : __reduce_min_sync(FULL, brk ? pos : kNoneHi);
  WarpFilt w;
  w.lb = lb;
  w.mb = w.ma = float_key(-CUDART_INF_F);
  if (PLAIN) {
    const bool none = d == 0 ? lb == kNoneLo : lb == kNoneHi;
    const bool before = none || (d == 0 ? pos > lb : pos < lb);
    w.ma = __reduce_max_sync(FULL, f.lo);
    w.mb = __reduce_max_sync(FULL, before ? f.lo : float_key(-CUDART_INF_F));
  }
  if (lane == 0) sm.wf[d][warp] = w;
}

// After the barrier: direction d's stop S (the first `break` in scan order; positions from it on
// are invalid) and the best certified lower bound M over the valid positions. Warp w holds
// positions 32w .. 32w + 31; the forward scan's position -1 (when `has_x`) comes first in its
// scan order. The maximal gain G* of the direction is at least M, so only positions whose upper
// bound reaches M can hold it; and any position passes min_gain_shift exactly when G* does.
template <bool PLAIN, int NW>
__device__ __forceinline__ void resolve_dir(const SearchSmemT<NW>& sm, int d, bool has_x, int* S, int32_t* M) {
  int s = d == 0 ? kNoneLo : kNoneHi;
#pragma unroll
  for (int w = 0; w < NW; ++w) s = d == 0 ? max(s, sm.wf[d][w].lb) : min(s, sm.wf[d][w].lb);
  if (d == 1 && has_x && sm.xf.lb == -1) s = -1;
  *S = s;
  int32_t m = float_key(-CUDART_INF_F);
  if (PLAIN) {
    const bool none = d == 0 ? s == kNoneLo : s == kNoneHi;
    if (d == 1 && has_x && s != -1) m = sm.xf.ma;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      const WarpFilt& f = sm.wf[d][w];
      const bool contains = !none && f.lb == s;
      const bool all_before = none || (d == 0 ? 32 * w > s : 32 * w + 31 < s);
      if (contains)
        m = max(m, f.mb);
      else if (all_before)
        m = max(m, f.ma);
    }
  }
  *M = m;
}

// !(gain <= mgs) without an f64 comparison.
__device__ __forceinline__ bool gain_passes(double gain, double mgs) {
  return dnan(gain) || dnan(mgs) || dkey(gain) > dkey(mgs);
}
__device__ __forceinline__ bool is_neg_inf(double x) {
  return (unsigned long long)__double_as_longlong(x) == 0xfff0000000000000ULL;
}

// Appends this thread's entry (when `push`) to direction d's queue, one shared atomic per warp.
template <int NW>
__device__ __forceinline__ void queue_push(SearchSmemT<NW>& sm, int d, bool push, const QEnt& e, int lane) {
  const unsigned bal = __ballot_sync(FULL, push);
  int base = 0;
  if (lane == 0 && bal) base = atomicAdd(&sm.qn[d], __popc(bal));
  base = __shfl_sync(FULL, base, 0);
  if (push) sm.q[d][base + __popc(bal & ((1u << lane) - 1u))] = e;
}

// Queue batches of 8 positions, four lanes per position: lanes 4k, 4k + 1 evaluate the left and
// right leaf gains of position k, lanes 4k + 2, 4k + 3 its left and right outputs (SidePart). An
// f64 instruction costs a scheduler the same whether one lane or 32 run it, so spreading a
// position's two gains and two outputs over four lanes (one division each, in the same
// instructions) shortens its instruction chain to a quarter of the work, and evaluating every
// queued position's outputs with its gain leaves none to evaluate after the arg-max. Batch k of direction d runs on warp
// d + 2 (k mod 4), so the first batches of the two directions run on two schedulers and longer
// queues spread over all four. One warp: its batches k0, k0 + 4, ...; their arg-max (highest gain,
// ties to the earliest position in scan order) with its SplitInfo, and whether any passed, into
// sm.pres[d][k0] / sm.psplit[d][k0]. (With NW warps, batch k runs on warp d + 2 (k mod NW / 2).)
template <int NW, typename SideOf>
__device__ __forceinline__ void eval_batches(SearchSmemT<NW>& sm, int d, int k0, int lane, double mgs, SideOf side_of) {
  DirBest r;
  r.key = kNoKey;
  r.ev.gain = -CUDART_INF;
  r.a = r.b = 0;
  r.t = d == 0 ? kNoneLo : kNoneHi;
  r.c = 0;
  int split = 0;
  const int n = sm.qn[d];
  const int k = lane >> 2, role = lane & 3;
  auto batch = [&](int b0) {
    // quads past the queue's end evaluate its last entry and discard the result: an all-zero
    // entry would send the whole warp through the f64 division's slow path (zero dividend, tiny
    // divisor), which costs more than the gain itself on this part
    const bool have = b0 + k < n;
    const QEnt e = sm.q[d][have ? b0 + k : n - 1];
    const SidePart sp = side_of(e, role);
    const int q0 = lane & ~3;
    const double gl = __shfl_sync(FULL, sp.val, q0);
    const double gr = __shfl_sync(FULL, sp.val, q0 | 1);
    double g = gl + gr;
    if (!have) g = -CUDART_INF;
    const bool passed = have && gain_passes(g, mgs);
    if (__any_sync(FULL, passed)) split = 1;
    const bool elig = passed && !dnan(g) && !is_neg_inf(g);  // NaN never wins
    const long long key = warp_max64(elig ? dkey(g) : kNoKey);
    if (key == kNoKey) return;
    const bool at = elig && dkey(g) == key;
    const int tb = d == 0 ? __reduce_max_sync(FULL, at ? (int)e.t : kNoneLo)
                          : __reduce_min_sync(FULL, at ? (int)e.t : kNoneHi);
    const int wl = __ffs(__ballot_sync(FULL, at && (int)e.t == tb)) - 1 & ~3;  // the quad's first lane
    Eval v;
    v.gain = __shfl_sync(FULL, g, wl);
    v.lsg = __shfl_sync(FULL, sp.sg, wl + 2);
    v.lsh = __shfl_sync(FULL, sp.sh, wl + 2);
    v.lo = __shfl_sync(FULL, sp.val, wl + 2);
    v.lc = __shfl_sync(FULL, sp.n, wl + 2);
    v.rsg = __shfl_sync(FULL, sp.sg, wl + 3);
    v.rsh = __shfl_sync(FULL, sp.sh, wl + 3);
    v.ro = __shfl_sync(FULL, sp.val, wl + 3);
    v.rc = __shfl_sync(FULL, sp.n, wl + 3);
    v.lint = v.rint = 0;
    const int64_t wa = __shfl_sync(FULL, e.a, wl), wb = __shfl_sync(FULL, e.b, wl);
    const int32_t wc = __shfl_sync(FULL, e.c, wl);
    if (key > r.key || (key == r.key && earlier(d, tb, r.t))) {
      r.key = key;
      r.t = tb;
      r.ev = v;
      r.a = wa;
      r.b = wb;
      r.c = wc;
    }
  };
  // the first batch outside the loop: the f64 gain evaluated inside a loop measured about twice
  // as slow as the same code in straight-line form
  constexpr int kLanes = NW / 2;  // batch lanes per direction
  if (8 * k0 < n) batch(8 * k0);
  for (int b0 = 8 * (k0 + kLanes); b0 < n; b0 += 8 * kLanes) batch(b0);
  if (lane == 0) {
    sm.pres[d][k0] = r;
    sm.psplit[d][k0] = split;
  }
}

// After the queues are filled (barrier 3): the NW warps evaluate the queue batches (warp w takes
// direction w & 1, batches w >> 1, (w >> 1) + NW / 2, ...). Barrier 4; then warp 0 combines the
// batch results of each direction into r / rs, the winner's SplitInfo included.
template <int NW, typename SideOf>
__device__ __forceinline__ void eval_queues(SearchSmemT<NW>& sm, int warp, int lane, double mgs, SideOf side_of,
                                            DirBest (&r)[2], int (&rs)[2]) {
  static_assert(NW >= 2 && NW <= 8 && NW % 2 == 0, "one batch lane of each direction per pair of warps");
  const int d = warp & 1, k0 = warp >> 1;
  if (k0 < NW / 2) eval_batches<NW>(sm, d, k0, lane, mgs, side_of);
  __syncthreads();
  if (warp != 0) return;
#pragma unroll
  for (int dd = 0; dd < 2; ++dd) {
    r[dd] = sm.pres[dd][0];
    rs[dd] = sm.psplit[dd][0];
#pragma unroll
    for (int k = 1; k < NW / 2; ++k) {
      const DirBest& x = sm.pres[dd][k];
      rs[dd] |= sm.psplit[dd][k];
      if (x.key != kNoKey && (x.key > r[dd].key || (x.key == r[dd].key && earlier(dd, x.t, r[dd].t)))) r[dd] = x;
    }
  }
}

__device__ __forceinline__ void store_cand(const Job& J, const Params& p, int side, int32_t leaf, int32_t f,
                                           const Cand& c) {
  J.cand[(size_t)leaf * p.F + f] = c;
  J.cgain[side * p.F + f] = c.gain;
  J.csplit[side * p.F + f] = (uint8_t)c.splittable;
  J.cthr[side * p.F + f] = c.threshold | ((uint32_t)(c.default_left != 0) << 31);
}

// The combination of the directions (feature_histogram.rs:240-357, :700-830): the reverse scan
// first, the forward scan replaces it only with a strictly larger gain; then the chosen threshold's
// SplitInfo (`eval_of(best, direction)`), the penalty and the feature's candidate record. Warp 0,
// every lane with the same values.
template <typename EvalOf>
__device__ __forceinline__ void finish_cand(const Job& J, const Params& p, const DevFeature& m, int side, int32_t leaf,
                                            int32_t f, const ScanGeom& G, double mgs, const DirBest (&r)[2],
                                            const int (&rs)[2], int lane, EvalOf eval_of) {
  const int nd = G.two ? 2 : 1;
  int sp = 0, ch = -1;
  double cgain = -CUDART_INF;
  for (int i = 0; i < nd; ++i) {
    sp |= rs[i];
    if (rs[i] && r[i].ev.gain > cgain + mgs) {
      ch = i;
      cgain = r[i].ev.gain - mgs;
    }
  }
  Cand c;
  cand_reset(&c, m.real, f);
  if (ch >= 0) {
    // field-wise selects keep the chosen direction in registers
    DirBest b;
    b.key = ch == 0 ? r[0].key : r[1].key;
    b.a = ch == 0 ? r[0].a : r[1].a;
    b.b = ch == 0 ? r[0].b : r[1].b;
    b.c = ch == 0 ? r[0].c : r[1].c;
    b.t = ch == 0 ? r[0].t : r[1].t;
    b.ev = ch == 0 ? r[0].ev : r[1].ev;
    const Eval e = eval_of(b, ch);
    const int32_t t = b.t;
    c.threshold = (uint32_t)(ch == 0 ? t - 1 + G.off : t + G.off);
    c.left_output = e.lo;
    c.left_count = e.lc;
    c.lsg = e.lsg;
    c.lsh = e.lsh;
    c.right_output = e.ro;
    c.right_count = e.rc;
    c.rsg = e.rsg;
    c.rsh = e.rsh;
    c.lint = e.lint;
    c.rint = e.rint;
    c.gain = cgain;
    c.default_left = ch == 0 ? 1 : 0;
  }
  if (nd == 1 && m.missing == 2) c.default_left = 0;
  c.gain *= m.penalty;
  c.splittable = sp;
  c.missing = m.missing;
  if (lane == 0) store_cand(J, p, side, leaf, f, c);
}

// FindBestThresholdInt for one (leaf, feature): feature_histogram.rs:673-830, scans :839-1142.
// Three barriers: the prefix scan (with the most-frequent-bin fix and the forward scan's start
// folded in), the stop / prefilter summaries, and the arg-max.
template <bool PLAIN, int NW>
__device__ void search_int(const Job& J, const Params& p, const SearchIn& si, const DevFeature& m, int side,
                           int32_t f, int32_t leaf, SearchSmemT<NW>& sm) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const LeafConst& C = si.C;
  const int64_t s_int = si.S0.int_sum;
  const int64_t l_int = side ? C.ls.int_sum : s_int;
  const size_t slot_stride = (size_t)p.T * p.B * TILE;
  const size_t feat_off = (size_t)(f / TILE) * p.B * TILE + (f % TILE);
  int64_t* pool = reinterpret_cast<int64_t*>(J.pool);
  int64_t* hs = pool + (size_t)si.sslot * slot_stride + feat_off;  // group bin 0 of the feature
  int64_t* hl = pool + (size_t)(side ? si.lslot : si.sslot) * slot_stride + feat_off;
  const bool fix = m.mfb > 0;  // offset 0: the slice holds every bin and the most frequent one is empty
  const bool in = t < m.len;
  // the smaller leaf's most-frequent entry is rewritten by its side-0 CTA; side 1 never reads it
  const IntPool pv = si.pre ? IntPool{si.sv, si.lv} : int_pool(J, p, m, side, f, si.sslot, si.lslot);
  const int64_t sv = pv.sv, lv = pv.lv;
  const ScanGeom G = scan_geom(m);
  if (t < 2) sm.qn[t] = 0;
  const bool skip_t = G.skip && t + G.off == m.default_bin;
  const bool acc_t = !skip_t && t <= G.tf_r;  // bin t is accumulated by the scans
  const int64_t v0 = side ? lv - sv : sv;     // before the most-frequent bin's fix
  // barrier 1: the packed prefix sums of the accumulated bins, plus the sum that fixes the
  // most-frequent bin (fix) or starts the forward scan outside the slice (fwd_rest; never both:
  // fix needs offset 0, fwd_rest offset 1). Packed arithmetic is exact componentwise.
  int64_t w = acc_t ? v0 : 0;
  int64_t P = warp_incl_scan(w, lane);
  const int64_t aux = warp_sum(fix ? sv : v0);
  if (lane == 31) sm.wi[0][warp] = P;
  if (lane == 0) sm.wi[1][warp] = aux;
  __syncthreads();
  int64_t T = 0, AUX = 0;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    const int64_t y = sm.wi[0][i];
    if (i < warp) P += y;
    T += y;
    AUX += sm.wi[1][i];
  }
  int64_t v = v0;
  if (fix) {
    const int64_t fixed = s_int - AUX;  // FixHistogram: the leaf total minus every other bin
    const int64_t delta = side ? -fixed : fixed;
    if (t == m.mfb) {
      v = v0 + delta;
      if (side == 0) hs[(size_t)(t + 1) * TILE] = fixed;
    }
    if (m.mfb <= G.tf_r && !(G.skip && m.mfb + G.off == m.default_bin)) {
      T += delta;
      if (t >= m.mfb) P += delta;
      if (t == m.mfb) w += delta;
    }
  }
  if (side && in) hl[(size_t)(t + 1) * TILE] = v;
  const int64_t base_f = G.fwd_rest ? l_int - AUX : 0;
  const int64_t tg = unpack_g(l_int), th = unpack_h(l_int);
  // reverse position t: right side = bins t .. tf_r; forward position t: left side = base_f plus
  // bins 0 .. t; the last thread also holds forward position -1 (left side = base_f)
  const int64_t right = T - (P - w);
  const int64_t left = base_f + P;
  const bool xpos = G.fwd_rest && t == 32 * NW - 1;
  const bool first0 = t >= 1 - G.off && acc_t && unpack_h(right) >= C.first_x;
  const bool brk0 = first0 && unpack_h(right) >= C.brk_x;
  const bool first1 = G.two && t <= G.t_end && !skip_t && unpack_h(left) >= C.first_x;
  const bool brk1 = first1 && unpack_h(left) >= C.brk_x;
  const bool firstx = xpos && unpack_h(base_f) >= C.first_x;
  const bool brkx = firstx && unpack_h(base_f) >= C.brk_x;
  const int64_t lg[2] = {tg - unpack_g(right), xpos ? unpack_g(base_f) : unpack_g(left)};
  const int64_t lh[2] = {th - unpack_h(right), xpos ? unpack_h(base_f) : unpack_h(left)};
  // barrier 2: stops and prefilter summaries
  Filt fl[2];
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const bool cand = d == 0 ? first0 : (first1 || firstx);
    Approx a{0.f, 0.f, true};
    if (PLAIN && cand) a = approx_int(lg[d], lh[d], tg, th, C.gsf, C.hsf, C.l2f);
    fl[d] = filt_of(cand, a, C);
  }
  publish_dir<PLAIN, NW>(sm, 0, brk0, t, fl[0], lane, warp);
  {
    Filt nat = fl[1];
    if (xpos) nat.lo = float_key(-CUDART_INF_F);  // the natural position 255 is never a candidate
    publish_dir<PLAIN, NW>(sm, 1, brk1, t, nat, lane, warp);
  }
  if (xpos) {
    WarpFilt x;
    x.lb = brkx ? -1 : kNoneHi;
    x.ma = x.mb = fl[1].lo;
    sm.xf = x;
  }
  __syncthreads();
  int S[2];
  int32_t M[2];
  resolve_dir<PLAIN, NW>(sm, 0, false, &S[0], &M[0]);
  resolve_dir<PLAIN, NW>(sm, 1, G.fwd_rest, &S[1], &M[1]);
  const bool valid[2] = {first0 && t > S[0], xpos ? (firstx && S[1] != -1) : (first1 && t < S[1])};
  DirBest r[2];
  int rs[2] = {0, 0};
  if (PLAIN) {
    // a position whose bin adds nothing repeats its scan predecessor (t + 1 reverse, t - 1 forward)
    const bool rep[2] = {w == 0 && t + 1 <= G.tf_r && !(G.skip && t + 1 + G.off == m.default_bin),
                         !xpos && w == 0 && ((t >= 1 && !(G.skip && t - 1 + G.off == m.default_bin)) ||
                                             (t == 0 && G.fwd_rest))};
    // barrier 3: the few positions that need their f64 gain; barrier 4: evaluated on the eight warps
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const bool exact = valid[d] && !rep[d] && (fl[d].unc || (fl[d].mp && fl[d].up >= M[d]));
      queue_push(sm, d, exact, QEnt{lg[d], lh[d], 0, (int16_t)(d == 0 || !xpos ? t : -1), (int16_t)d}, lane);
    }
    __syncthreads();
    const double gs = C.gs, hsc = C.hs;
    eval_queues(
        sm, warp, lane, C.mgs,
        [&](const QEnt& e, int role) { return int_side(p, e.a, e.b, tg, th, gs, hsc, C.cnt_factor, role); }, r, rs);
    if (warp != 0) return;
  } else {
    // every valid position evaluates its own f64 gain; barrier 3: the arg-max
    double gain[2];
    bool split[2], elig[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      gain[d] = -CUDART_INF;
      if (valid[d])
        gain[d] = int_split_gain(p, lg[d], lh[d], tg, th, C.gs, C.hs, C.cnt_factor, C.parent, false);
      const bool passed = valid[d] && gain_passes(gain[d], C.mgs);
      split[d] = passed;
      elig[d] = passed && !dnan(gain[d]) && !is_neg_inf(gain[d]);  // NaN never wins
    }
    warp_best(0, elig[0], gain[0], t, lg[0], lh[0], 0, lane, &sm.wb[0][warp]);
    warp_best(1, elig[1], gain[1], xpos ? -1 : t, lg[1], lh[1], 0, lane, &sm.wb[1][warp]);
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const int ws = __any_sync(FULL, split[d]);
      if (lane == 0) sm.spl[d][warp] = ws;
    }
    __syncthreads();
    if (warp != 0) return;
    combine_best(sm, lane, r, rs);
  }
  // FindBestThresholdInt's combination of the directions (feature_histogram.rs:700-830)
  finish_cand(J, p, m, side, leaf, f, G, C.mgs, r, rs, lane, [&](const DirBest& b, int d) {
    (void)d;
    if (PLAIN) {  // evaluated with the gain
      Eval v = b.ev;
      v.lint = (int64_t)(((uint64_t)b.a << 32) | ((uint64_t)b.b & 0xffffffffull));
      v.rint = (int64_t)(((uint64_t)(tg - b.a) << 32) | ((uint64_t)(th - b.b) & 0xffffffffull));
      return v;
    }
    return eval_int(p, b.a, b.b, tg, th, C.gs, C.hs, C.cnt_factor, C.parent, b.ev.gain, lane);
  });
}

// FindBestThreshold (float) for one (leaf, feature): feature_histogram.rs:219-357, scans
// :363-663. f64 (grad, hess) sums and row counts estimated per bin as round_int(hess *
// cnt_factor); the forward scan uses prefix sums, the reverse scan suffix sums (accumulated from
// the top bin down, not derived by subtraction).
template <bool PLAIN, int NW>
__device__ void search_float(const Job& J, const Params& p, const SearchIn& si, const DevFeature& m, int side,
                             int32_t f, int32_t leaf, SearchSmemT<NW>& sm) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const LeafConst& C = si.C;
  const LeafSum& S0 = si.S0;
  const int32_t num_data = side ? C.ls.num_data : S0.num_data;
  const size_t slot_stride = (size_t)p.T * p.B * TILE;
  const size_t feat_off = (size_t)(f / TILE) * p.B * TILE + (f % TILE);
  double2* pool = reinterpret_cast<double2*>(J.pool);
  double2* hs = pool + (size_t)si.sslot * slot_stride + feat_off;
  double2* hl = pool + (size_t)(side ? si.lslot : si.sslot) * slot_stride + feat_off;
  const double2 zero = make_double2(0.0, 0.0);
  const bool fix = m.mfb > 0;
  const bool in = t < m.len;
  double2 sv = (in && !(fix && t == m.mfb)) ? hs[(size_t)(t + 1) * TILE] : zero;
  const double2 lv = (side && in) ? hl[(size_t)(t + 1) * TILE] : zero;
  const ScanGeom G = scan_geom(m);
  if (t < 2) sm.qn[t] = 0;
  const double sum_g = C.sum_g, sum_h = C.sum_h;
  if (fix) {  // one barrier for both sums
    const double ag = warp_sum(sv.x), ah = warp_sum(sv.y);
    if (lane == 0) {
      sm.wd[0][warp] = ag;
      sm.wd[1][warp] = ah;
    }
    __syncthreads();
    double tg = 0.0, th = 0.0;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      tg += sm.wd[0][i];
      th += sm.wd[1][i];
    }
    if (t == m.mfb) {
      sv = make_double2(S0.sg - tg, S0.sh - th);
      if (side == 0) hs[(size_t)(t + 1) * TILE] = sv;
    }
  }
  const double2 v = side ? make_double2(lv.x - sv.x, lv.y - sv.y) : sv;
  if (side && in) hl[(size_t)(t + 1) * TILE] = v;
  const int32_t cn = in ? round_int(v.y * C.cnt_factor) : 0;
  // barrier: prefix sums (forward), suffix sums over bins <= tf_r (reverse) and, when the forward
  // scan starts outside the slice, the slice totals
  const bool skip_t = G.skip && t + G.off == m.default_bin;
  const double wg = skip_t ? 0.0 : v.x, wh = skip_t ? 0.0 : v.y;
  const int32_t wc = skip_t ? 0 : cn;
  const bool rin = t <= G.tf_r;
  double pg = warp_incl_scan(wg, lane), ph = warp_incl_scan(wh, lane);
  int32_t pc = warp_incl_scan(wc, lane);
  double rg = warp_incl_scan_down(rin ? wg : 0.0, lane), rh = warp_incl_scan_down(rin ? wh : 0.0, lane);
  int32_t rc = warp_incl_scan_down(rin ? wc : 0, lane);
  if (lane == 31) {
    sm.wd[2][warp] = pg;
    sm.wd[3][warp] = ph;
    sm.wc[0][warp] = pc;
  }
  if (lane == 0) {
    sm.wd[4][warp] = rg;
    sm.wd[5][warp] = rh;
    sm.wc[1][warp] = rc;
  }
  if (G.fwd_rest) {
    const double ug = warp_sum(v.x), uh = warp_sum(v.y);
    const int32_t uc = warp_sum(cn);
    if (lane == 0) {
      sm.wd[6][warp] = ug;
      sm.wd[7][warp] = uh;
      sm.wc[2][warp] = uc;
    }
  }
  __syncthreads();
  // forward scan start: nothing (with kEpsilon hessian) or everything outside the slice
  double bg = 0.0, bh = BK_EPS;
  int32_t bc = 0;
  {
    double og = 0.0, oh = 0.0, sg_ = 0.0, sh_ = 0.0, ug = 0.0, uh = 0.0;
    int32_t oc = 0, sc = 0, uc = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      if (i < warp) {
        og += sm.wd[2][i];
        oh += sm.wd[3][i];
        oc += sm.wc[0][i];
      }
    }
#pragma unroll
    for (int i = NW - 1; i >= 0; --i) {
      if (i > warp) {
        sg_ += sm.wd[4][i];
        sh_ += sm.wd[5][i];
        sc += sm.wc[1][i];
      }
    }
    if (G.fwd_rest) {
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        ug += sm.wd[6][i];
        uh += sm.wd[7][i];
        uc += sm.wc[2][i];
      }
      bg = sum_g - ug;
      bh = (sum_h - BK_EPS) - uh;
      bc = num_data - uc;
    }
    pg = bg + (pg + og);
    ph = bh + (ph + oh);
    pc = bc + (pc + oc);
    rg = rg + sg_;
    rh = BK_EPS + (rh + sh_);
    rc = rc + sc;
  }
  // reverse position t: right side (rg, rh, rc); forward position t: left side (pg, ph, pc); the
  // last thread holds forward position -1 when the scan starts outside the slice
  const bool xpos = G.fwd_rest && t == 32 * NW - 1;
  const bool first0 = t >= 1 - G.off && rin && !skip_t && !(rc < p.min_data || rh < p.min_hess);
  const bool brk0 = first0 && (num_data - rc < p.min_data || sum_h - rh < p.min_hess);
  const bool first1 = G.two && t <= G.t_end && !skip_t && !(pc < p.min_data || ph < p.min_hess);
  const bool brk1 = first1 && (num_data - pc < p.min_data || sum_h - ph < p.min_hess);
  const bool firstx = xpos && !(bc < p.min_data || bh < p.min_hess);
  const bool brkx = firstx && (num_data - bc < p.min_data || sum_h - bh < p.min_hess);
  const double fg = xpos ? bg : pg, fh = xpos ? bh : ph;
  const int32_t fc = xpos ? bc : pc;
  // left / right sums of both positions
  const double slg[2] = {sum_g - rg, fg}, slh[2] = {sum_h - rh, fh};
  const double srg[2] = {rg, sum_g - fg}, srh[2] = {rh, sum_h - fh};
  const int32_t lc[2] = {num_data - rc, fc}, rcn[2] = {rc, num_data - fc};
  Filt fl[2];
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    const bool cand = d == 0 ? first0 : (first1 || firstx);
    Approx a{0.f, 0.f, true};
    if (PLAIN && cand)
      a = approx_from((float)slg[d], __fadd_rn((float)slh[d], C.l2f), (float)srg[d], __fadd_rn((float)srh[d], C.l2f));
    fl[d] = filt_of(cand, a, C);
  }
  publish_dir<PLAIN, NW>(sm, 0, brk0, t, fl[0], lane, warp);
  {
    Filt nat = fl[1];
    if (xpos) nat.lo = float_key(-CUDART_INF_F);
    publish_dir<PLAIN, NW>(sm, 1, brk1, t, nat, lane, warp);
  }
  if (xpos) {
    WarpFilt x;
    x.lb = brkx ? -1 : kNoneHi;
    x.ma = x.mb = fl[1].lo;
    sm.xf = x;
  }
  __syncthreads();
  int S[2];
  int32_t M[2];
  resolve_dir<PLAIN, NW>(sm, 0, false, &S[0], &M[0]);
  resolve_dir<PLAIN, NW>(sm, 1, G.fwd_rest, &S[1], &M[1]);
  const bool valid[2] = {first0 && t > S[0], xpos ? (firstx && S[1] != -1) : (first1 && t < S[1])};
  DirBest r[2];
  int rs[2] = {0, 0};
  // carried per position: the accumulated side's sums (reverse: right, forward: left)
  const int64_t ca[2] = {__double_as_longlong(rg), __double_as_longlong(fg)};
  const int64_t cb[2] = {__double_as_longlong(rh), __double_as_longlong(fh)};
  const int32_t cc[2] = {rc, fc};
  auto gain_of = [&](const QEnt& e) {
    const double ag = __longlong_as_double(e.a), ah = __longlong_as_double(e.b);
    if (e.d == 0)  // reverse: (ag, ah, c) is the right side
      return split_gains(p, sum_g - ag, sum_h - ah, ag, ah, num_data - e.c, e.c, C.parent);
    return split_gains(p, ag, ah, sum_g - ag, sum_h - ah, e.c, num_data - e.c, C.parent);
  };
  if (PLAIN) {
    // a position whose bin adds nothing repeats its scan predecessor (t + 1 reverse, t - 1 forward)
    const bool empty = wg == 0.0 && wh == 0.0 && wc == 0;
    const bool rep[2] = {empty && t + 1 <= G.tf_r && !(G.skip && t + 1 + G.off == m.default_bin),
                         !xpos && empty && ((t >= 1 && !(G.skip && t - 1 + G.off == m.default_bin)) ||
                                            (t == 0 && G.fwd_rest))};
    // barrier 3: the few positions that need their f64 gain; barrier 4: evaluated on the eight warps
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const bool exact = valid[d] && !rep[d] && (fl[d].unc || (fl[d].mp && fl[d].up >= M[d]));
      queue_push(sm, d, exact, QEnt{ca[d], cb[d], cc[d], (int16_t)(d == 0 || !xpos ? t : -1), (int16_t)d}, lane);
    }
    __syncthreads();
    eval_queues(
        sm, warp, lane, C.mgs,
        [&](const QEnt& e, int role) {
          return float_side(p, e.d, __longlong_as_double(e.a), __longlong_as_double(e.b), e.c, sum_g, sum_h,
                            num_data, role);
        },
        r, rs);
    if (warp != 0) return;
  } else {
    double gain[2];
    bool split[2], elig[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      gain[d] = -CUDART_INF;
      if (valid[d]) gain[d] = split_gains(p, slg[d], slh[d], srg[d], srh[d], lc[d], rcn[d], C.parent);
      const bool passed = valid[d] && gain_passes(gain[d], C.mgs);
      split[d] = passed;
      elig[d] = passed && !dnan(gain[d]) && !is_neg_inf(gain[d]);
    }
    warp_best(0, elig[0], gain[0], t, ca[0], cb[0], cc[0], lane, &sm.wb[0][warp]);
    warp_best(1, elig[1], gain[1], xpos ? -1 : t, ca[1], cb[1], cc[1], lane, &sm.wb[1][warp]);
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const int ws = __any_sync(FULL, split[d]);
      if (lane == 0) sm.spl[d][warp] = ws;
    }
    __syncthreads();
    if (warp != 0) return;
    combine_best(sm, lane, r, rs);
  }
  // FindBestThreshold's combination of the directions (feature_histogram.rs:240-357)
  finish_cand(J, p, m, side, leaf, f, G, C.mgs, r, rs, lane, [&](const DirBest& b, int d) {
    if (PLAIN) return b.ev;  // evaluated with the gain
    return eval_float(p, d, __longlong_as_double(b.a), __longlong_as_double(b.b), b.c, sum_g, sum_h, num_data,
                      C.parent, b.ev.gain, lane);
  });
}

// ---- categorical features (feature_histogram.rs:1328-1886) ----
// One CTA per (leaf side, feature) as for numerical features; thread t holds slice index t. The
// histogram slice is loaded, fixed and (larger side) derived by subtraction exactly as the
// numerical searches do, so the pool holds the same values afterwards. Then:
//   one-hot (num_bin <= max_cat_to_onehot): every category's split against the rest is evaluated
//     by its own thread; the first best in category order wins;
//   sorted: the categories with enough data are ranked by grad / (hess + cat_smooth) (a stable
//     rank over order-preserving integer keys, ties by category), one thread per direction walks
//     the reference's sequential scan (its sums, counts, skips and breaks do not depend on the
//     gains) and queues the positions that need a gain, which the CTA then evaluates in parallel;
//     the first best in scan order (ascending direction first) wins.
// Gains and outputs use lambda_l2 + cat_l2 in the sorted form, as the reference does.
constexpr int kCatQueue = kSearchThreads / 2;  // queued positions per direction: max_num_cat <= 128

// The categorical search's shared memory, overlaid on the numerical search's (a CTA runs one or
// the other). V: int64_t (quantized, integer sums) or double (float path).
template <typename V>
struct CatSmem {
  V a[kSearchThreads], b[kSearchThreads];  // per-bin gradient / hessian sums
  int32_t cnt[kSearchThreads];
  long long key[kSearchThreads];
  int16_t sorted[kSearchThreads];
  V qa[2][kCatQueue], qb[2][kCatQueue];    // queued positions: the accumulated left side's sums
  int32_t qlc[2][kCatQueue], qi[2][kCatQueue];
  int32_t qn[2];
  long long wk[kSearchWarps];
  int32_t wo[kSearchWarps], wsp[kSearchWarps];
  int64_t wi[kSearchWarps];
  double wd[2][kSearchWarps];
  double best_gain;
};

__device__ __forceinline__ long long cat_block_max(long long v, long long* w, int lane, int warp) {
  v = warp_max64(v);
  if (lane == 0) w[warp] = v;
  __syncthreads();
  long long r = w[0];
#pragma unroll
  for (int i = 1; i < kSearchWarps; ++i) r = w[i] > r ? w[i] : r;
  __syncthreads();
  return r;
}

__device__ __forceinline__ int32_t cat_block_min(int32_t v, int32_t* w, int lane, int warp) {
  v = __reduce_min_sync(FULL, v);
  if (lane == 0) w[warp] = v;
  __syncthreads();
  int32_t r = w[0];
#pragma unroll
  for (int i = 1; i < kSearchWarps; ++i) r = w[i] < r ? w[i] : r;
  __syncthreads();
  return r;
}

__device__ __forceinline__ int32_t cat_block_or(int32_t v, int32_t* w, int lane, int warp) {
  v = (int32_t)__reduce_or_sync(FULL, (unsigned)v);
  if (lane == 0) w[warp] = v;
  __syncthreads();
  int32_t r = 0;
#pragma unroll
  for (int i = 0; i < kSearchWarps; ++i) r |= w[i];
  __syncthreads();
  return r;
}

template <bool QUANT>
__device__ void search_cat(const Job& J, const Params& p, const SearchIn& si, const DevFeature& m, int side,
                           int32_t f, int32_t leaf, SearchSmem& sm) {
  using V = typename std::conditional<QUANT, int64_t, double>::type;
  static_assert(sizeof(CatSmem<V>) <= sizeof(SearchSmem), "the categorical search fits the search's shared memory");
  CatSmem<V>& cs = *reinterpret_cast<CatSmem<V>*>(&sm);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const LeafConst& C = si.C;
  const LeafSum& S0 = si.S0;
  const LeafSum& SL = C.ls;
  const int32_t num_data = SL.num_data;
  const size_t slot_stride = (size_t)p.T * p.B * TILE;
  const size_t feat_off = (size_t)(f / TILE) * p.B * TILE + (f % TILE);
  const bool fix = m.mfb > 0;
  const bool in = t < m.len;
  // -- the slice: FixHistogram of the smaller leaf, the larger as parent minus smaller (serial.rs:
  //    1407-1437, 2205-2238), written back exactly as the numerical searches write it --
  if (QUANT) {
    int64_t* pool = reinterpret_cast<int64_t*>(J.pool);
    int64_t* hs = pool + (size_t)si.sslot * slot_stride + feat_off;
    int64_t* hl = pool + (size_t)(side ? si.lslot : si.sslot) * slot_stride + feat_off;
    const int64_t sv = (in && !(fix && t == m.mfb)) ? hs[(size_t)(t + 1) * TILE] : 0;
    const int64_t lv = (side && in) ? hl[(size_t)(t + 1) * TILE] : 0;
    int64_t v = side ? lv - sv : sv;
    if (fix) {
      const int64_t a = warp_sum(sv);
      if (lane == 0) cs.wi[warp] = a;
      __syncthreads();
      int64_t aux = 0;
#pragma unroll
      for (int i = 0; i < kSearchWarps; ++i) aux += cs.wi[i];
      const int64_t fixed = S0.int_sum - aux;  // the leaf total minus every other bin
      if (t == m.mfb) {
        v += side ? -fixed : fixed;
        if (side == 0) hs[(size_t)(t + 1) * TILE] = fixed;
      }
    }
    if (side && in) hl[(size_t)(t + 1) * TILE] = v;
    cs.a[t] = in ? unpack_g(v) : 0;
    cs.b[t] = in ? unpack_h(v) : 0;
    cs.cnt[t] = in ? round_int((double)unpack_h(v) * C.cnt_factor) : 0;
  } else {
    double2* pool = reinterpret_cast<double2*>(J.pool);
    double2* hs = pool + (size_t)si.sslot * slot_stride + feat_off;
    double2* hl = pool + (size_t)(side ? si.lslot : si.sslot) * slot_stride + feat_off;
    const double2 zero = make_double2(0.0, 0.0);
    double2 sv = (in && !(fix && t == m.mfb)) ? hs[(size_t)(t + 1) * TILE] : zero;
    const double2 lv = (side && in) ? hl[(size_t)(t + 1) * TILE] : zero;
    if (fix) {
      const double ag = warp_sum(sv.x), ah = warp_sum(sv.y);
      if (lane == 0) {
        cs.wd[0][warp] = ag;
        cs.wd[1][warp] = ah;
      }
      __syncthreads();
      double tg = 0.0, th = 0.0;
#pragma unroll
      for (int i = 0; i < kSearchWarps; ++i) {
        tg += cs.wd[0][i];
        th += cs.wd[1][i];
      }
      if (t == m.mfb) {
        sv = make_double2(S0.sg - tg, S0.sh - th);
        if (side == 0) hs[(size_t)(t + 1) * TILE] = sv;
      }
    }
    const double2 v = side ? make_double2(lv.x - sv.x, lv.y - sv.y) : sv;
    if (side && in) hl[(size_t)(t + 1) * TILE] = v;
    cs.a[t] = in ? v.x : 0.0;
    cs.b[t] = in ? v.y : 0.0;
    cs.cnt[t] = in ? round_int(v.y * C.cnt_factor) : 0;
  }
  if (t < 2) cs.qn[t] = 0;
  __syncthreads();
  // -- the leaf's totals and min_gain_shift (feature_histogram.rs:1347-1386, :1614-1665) --
  const int64_t l_int = side ? SL.int_sum : S0.int_sum;
  const int64_t tgi = unpack_g(l_int), thi = unpack_h(l_int);
  const double gs = C.gs, hsc = C.hs;
  const double sum_g = C.sum_g, sum_h = C.sum_h;  // float path: sum_h includes 2 kEpsilon
  const double mgs =
      p.use_smooth ? leaf_gain_given_output(p.use_l1, sum_g, sum_h, p, C.parent) + p.min_gain : C.mgs;
  const int32_t bin_start = 1 - m.offset, bin_end = m.num_bin - m.offset;
  const bool onehot = m.num_bin <= p.max_cat_to_onehot;
  Params pl = p;
  int32_t best_dir = 0, best_i = -1, used_bin = 0, sp = 0;
  double best_gain = -CUDART_INF;
  // the chosen position's left side
  double blg = 0.0, blh = 0.0;
  int64_t big = 0, bih = 0;
  int32_t blc = 0;
  if (onehot) {
    // -- one category against the rest, thread t = category t --
    bool pass = false;
    double gain = -CUDART_INF;
    if (t >= bin_start && t < bin_end) {
      const int32_t cnt = cs.cnt[t];
      if (QUANT) {
        const int64_t ig = (int64_t)cs.a[t], ih = (int64_t)cs.b[t];
        const double h = (double)ih * hsc;
        const int32_t other_cnt = num_data - cnt;
        const double other_h = (double)(thi - ih) * hsc;
        if (!(cnt < p.min_data || h < p.min_hess) && other_cnt >= p.min_data && !(other_h < p.min_hess)) {
          const double g = (double)ig * gs, other_g = (double)(tgi - ig) * gs;
          gain = split_gains(pl, other_g, other_h, g, h, other_cnt, cnt, C.parent);
          pass = gain > mgs;
        }
      } else {
        const double g = (double)cs.a[t], h = (double)cs.b[t];
        const int32_t other_cnt = num_data - cnt;
        const double other_h = sum_h - h - BK_EPS;
        if (!(cnt < p.min_data || h < p.min_hess) && other_cnt >= p.min_data && !(other_h < p.min_hess)) {
          const double other_g = sum_g - g;
          gain = split_gains(pl, other_g, other_h, g, h + BK_EPS, other_cnt, cnt, C.parent);
          pass = gain > mgs;
        }
      }
    }
    sp = cat_block_or(pass ? 1 : 0, cs.wsp, lane, warp);
    const long long k = cat_block_max(pass ? dkey(gain) : kNoKey, cs.wk, lane, warp);
    if (k != kNoKey) {
      // the first category (in order) with the best gain
      const int32_t first = cat_block_min(pass && dkey(gain) == k ? t : 0x7fffffff, cs.wo, lane, warp);
      if (t == first) cs.best_gain = gain;
      __syncthreads();
      best_gain = cs.best_gain;
      best_i = first;
      blc = cs.cnt[first];
      if (QUANT) {
        big = (int64_t)cs.a[first];
        bih = (int64_t)cs.b[first];
      } else {
        blg = (double)cs.a[first];
        blh = (double)cs.b[first] + BK_EPS;
      }
    }
    if (warp != 0) return;
  } else {
    // -- the categories with enough data, ranked by grad / (hess + cat_smooth) --
    const bool elig = t >= bin_start && t < bin_end && (double)cs.cnt[t] >= p.cat_smooth;
    double ctr = 0.0;
    if (elig) {
      if (QUANT) ctr = ((double)cs.a[t] * gs) / ((double)cs.b[t] * hsc + p.cat_smooth);
      else ctr = (double)cs.a[t] / ((double)cs.b[t] + p.cat_smooth);
    }
    cs.key[t] = elig ? dkey(ctr) : kNoKey;
    const int32_t ne = __popc(__ballot_sync(FULL, elig));
    if (lane == 0) cs.wo[warp] = ne;
    __syncthreads();
    used_bin = 0;
#pragma unroll
    for (int i = 0; i < kSearchWarps; ++i) used_bin += cs.wo[i];
    if (elig) {
      const long long kt = cs.key[t];
      int32_t rank = 0;
      for (int u = 0; u < kSearchThreads; ++u) {
        const long long ku = cs.key[u];
        rank += (ku != kNoKey && (ku < kt || (ku == kt && u < t))) ? 1 : 0;
      }
      cs.sorted[rank] = (int16_t)t;
    }
    pl.l2 = p.l2 + p.cat_l2;
    __syncthreads();
    const int32_t max_num_cat = min(p.max_cat_threshold, (used_bin + 1) / 2);
    // -- the sequential scans, one thread per direction (warp 0 ascending, warp 1 descending) --
    if ((t == 0 || t == 32) && used_bin > 0) {
      const int d = t == 0 ? 0 : 1;
      const int dir = d == 0 ? 1 : -1;
      int32_t pos = d == 0 ? 0 : used_bin - 1, cnt_group = 0, left_cnt = 0, q = 0;
      double lg = 0.0, lh = BK_EPS;
      int64_t lig = 0, lih = 0;
      for (int32_t i = 0; i < used_bin && i < max_num_cat; ++i) {
        const int32_t c = cs.sorted[pos];
        pos += dir;
        const int32_t cnt = cs.cnt[c];
        left_cnt += cnt;
        cnt_group += cnt;
        double lhv;
        if (QUANT) {
          lig += (int64_t)cs.a[c];
          lih += (int64_t)cs.b[c];
          lhv = (double)lih * hsc;
        } else {
          lg += (double)cs.a[c];
          lh += (double)cs.b[c];
          lhv = lh;
        }
        if (left_cnt < p.min_data || lhv < p.min_hess) continue;
        const int32_t right_cnt = num_data - left_cnt;
        if (right_cnt < p.min_data || right_cnt < p.min_data_per_group) break;
        const double rhv = QUANT ? (double)(thi - lih) * hsc : sum_h - lh;
        if (rhv < p.min_hess) break;
        if (cnt_group < p.min_data_per_group) continue;
        cnt_group = 0;
        if (q < kCatQueue) {
          cs.qa[d][q] = QUANT ? (V)lig : (V)lg;
          cs.qb[d][q] = QUANT ? (V)lih : (V)lh;
          cs.qlc[d][q] = left_cnt;
          cs.qi[d][q] = i;
          ++q;
        }
      }
      cs.qn[d] = q;
    }
    __syncthreads();
    // -- the queued gains, one thread each: direction 0 on threads 0..127, direction 1 on 128..255 --
    const int d = t >> 7, j = t & 127;
    bool pass = false;
    double gain = -CUDART_INF;
    if (j < cs.qn[d]) {
      const int32_t lc = cs.qlc[d][j], rc = num_data - lc;
      if (QUANT) {
        const int64_t lig = (int64_t)cs.qa[d][j], lih = (int64_t)cs.qb[d][j];
        const double lg = (double)lig * gs, lh = (double)lih * hsc;
        const double rg = (double)(tgi - lig) * gs, rh = (double)(thi - lih) * hsc;
        gain = split_gains(pl, lg, lh, rg, rh, lc, rc, C.parent);
      } else {
        const double lg = (double)cs.qa[d][j], lh = (double)cs.qb[d][j];
        gain = split_gains(pl, lg, lh, sum_g - lg, sum_h - lh, lc, rc, C.parent);
      }
      pass = gain > mgs;
    }
    sp = cat_block_or(pass ? 1 : 0, cs.wsp, lane, warp);
    const long long k = cat_block_max(pass ? dkey(gain) : kNoKey, cs.wk, lane, warp);
    if (k != kNoKey) {
      // scan order: direction 0 before direction 1, then the position
      const int32_t first = cat_block_min(pass && dkey(gain) == k ? t : 0x7fffffff, cs.wo, lane, warp);
      best_dir = first >> 7;
      const int32_t bj = first & 127;
      best_i = cs.qi[best_dir][bj];
      if (QUANT) {
        big = (int64_t)cs.qa[best_dir][bj];
        bih = (int64_t)cs.qb[best_dir][bj];
      } else {
        blg = (double)cs.qa[best_dir][bj];
        blh = (double)cs.qb[best_dir][bj];
      }
      blc = cs.qlc[best_dir][bj];
      if (t == first) cs.best_gain = gain;
      __syncthreads();
      best_gain = cs.best_gain;
    }
    if (warp != 0) return;
  }
  // -- warp 0: the SplitInfo of the chosen position (feature_histogram.rs:1537-1598, :1828-1886) --
  Cand c;
  cand_reset(&c, m.real, f);
  c.default_left = 0;
  c.categorical = 1;
  uint32_t word = 0u;  // lane w: word w of the left bins' bitset
  if (sp && best_i >= 0) {
    if (QUANT) {
      const double lg = (double)big * gs, lh = (double)bih * hsc;
      const int64_t rig = tgi - big, rih = thi - bih;
      const double rg = (double)rig * gs, rh = (double)rih * hsc;
      const int32_t lc = round_int((double)bih * C.cnt_factor), rc = round_int((double)rih * C.cnt_factor);
      c.left_output = split_output(pl, lg, lh, lc, C.parent);
      c.right_output = split_output(pl, rg, rh, rc, C.parent);
      c.left_count = lc;
      c.right_count = rc;
      c.lsg = lg;
      c.lsh = lh;
      c.rsg = rg;
      c.rsh = rh;
      c.lint = (int64_t)(((uint64_t)big << 32) | ((uint64_t)bih & 0xffffffffULL));
      c.rint = (int64_t)(((uint64_t)rig << 32) | ((uint64_t)rih & 0xffffffffULL));
    } else {
      c.left_output = split_output(pl, blg, blh, blc, C.parent);
      c.right_output = split_output(pl, sum_g - blg, sum_h - blh, num_data - blc, C.parent);
      c.left_count = blc;
      c.right_count = num_data - blc;
      c.lsg = blg;
      c.lsh = blh - BK_EPS;
      c.rsg = sum_g - blg;
      c.rsh = sum_h - blh - BK_EPS;
    }
    c.gain = best_gain - mgs;
    // the bins that go left: the category itself (one-hot) or the first best_i + 1 categories of
    // the chosen scan direction; lane w collects word w of the bitset
    if (onehot) {
      const uint32_t b = (uint32_t)(best_i + m.offset);
      if ((int)(b >> 5) == lane) word |= 1u << (b & 31);
    } else {
      for (int32_t i = 0; i <= best_i; ++i) {
        const int32_t pos = best_dir == 0 ? i : used_bin - 1 - i;
        const uint32_t b = (uint32_t)(cs.sorted[pos] + m.offset);
        if ((int)(b >> 5) == lane) word |= 1u << (b & 31);
      }
    }
  }
  c.gain *= m.penalty;
  c.splittable = sp;
  c.missing = m.missing;
  if (lane == 0) store_cand(J, p, side, leaf, f, c);
  if (lane < 8) cand_cat_bits(J, p, leaf, f)[lane] = word;
}

// One CTA per (feature, side): blockIdx.x = 2 * feature + side (0 = smaller leaf). With `decide`,
// the last CTA to finish runs the fold / arg-max and records the split; otherwise the single-pass
// partition that follows decides it.
// NW warps per CTA: 8 for features of up to 256 group bins; 2 (64 threads) when every feature
// has at most 64, so a CTA holds what a small-bin feature needs and four times as many CTAs fit
// on an SM. Only NW = 8 takes categorical features and the stable path's last-CTA decision
// (both use 256 threads); the host picks NW accordingly.
// post: the histogram launch before this one applied a single-pass split's bookkeeping.
template <bool PLAIN, bool QUANT, int NW>
__global__ void __launch_bounds__(32 * NW) k_search(const JobTable jobs, Params p,
                                                    const DevFeature* __restrict__ feats, int clear_par,
                                                    int decide, int post) {
  __shared__ SearchSmemT<NW> sm;
  __shared__ int last;
  __shared__ Decision dec;
  const int side = (int)(blockIdx.x & 1u);
  const int f = (int)(blockIdx.x >> 1);
  const DevFeature m = feats[f];  // static: loaded while the histogram launch finishes
  const Job& J = jobs.job[blockIdx.z];
  JobState* st = J.st;
  // The two leaves' pool slots, read while the histogram launch finishes: this launch starts only
  // after every histogram CTA has passed its own wait, so the launches before that one are
  // complete. After a single-pass split the smaller child takes the slot the decision recorded
  // and the larger one keeps its parent's (split_pslot); otherwise the state's slots were written
  // before the histogram launch started. The state's own slots, read after the wait, confirm them
  // (a mismatch reloads); clamped, an early slot only ever addresses the pool.
  int32_t pre_s = -1, pre_l = -1;
  if (QUANT && !m.cat) {
    pre_s = __ldcg(post ? &st->split_sslot : &st->smaller_slot);
    pre_l = __ldcg(post ? &st->split_pslot : &st->larger_slot);
  }
  griddep_wait();
  // the partition may be scheduled now: its CTAs read their static data while this search runs,
  // and wait for its completion before reading anything it writes
  griddep_launch();
  if (clear_par >= 0 && blockIdx.x == 0 && threadIdx.x < 2) {
    // the single-pass partition counter pair of the split after next: its last reader, the
    // histogram launch before this one, has finished
    st->pcnt[clear_par][threadIdx.x] = 0;
  }
  // one round of independent loads: the state, the feature's flag, both leaves' constants and
  // (integer search) this thread's pool entries at the early slots
  const int32_t stop = st->stop, do_search = st->do_search;
  const int32_t leaf = side ? st->larger_leaf : st->smaller_leaf;
  const uint8_t used = J.used[f];
  SearchIn si;
  si.sslot = st->smaller_slot;
  si.lslot = st->larger_slot;
  si.C = J.lconst[side];
  si.S0 = side ? J.lconst[0].ls : si.C.ls;
  si.pre = false;
  if (QUANT && !m.cat) {
    const bool ok_s = (unsigned)pre_s < (unsigned)p.num_leaves, ok_l = (unsigned)pre_l < (unsigned)p.num_leaves;
    const IntPool pv = int_pool(J, p, m, side, f, ok_s ? pre_s : 0, ok_l ? pre_l : 0);
    si.sv = pv.sv;
    si.lv = pv.lv;
    si.pre = ok_s && pre_s == si.sslot && (side == 0 || (ok_l && pre_l == si.lslot));
  }
  if (stop) return;  // uniform over the grid
  if (do_search && used && leaf >= 0) {  // uniform over the CTA
    if constexpr (NW == kSearchWarps) {
      if (m.cat) {
        search_cat<QUANT>(J, p, si, m, side, f, leaf, sm);
      } else if (QUANT) {
        search_int<PLAIN>(J, p, si, m, side, f, leaf, sm);
      } else {
        search_float<PLAIN>(J, p, si, m, side, f, leaf, sm);
      }
    } else {
      if (QUANT) search_int<PLAIN>(J, p, si, m, side, f, leaf, sm);
      else search_float<PLAIN>(J, p, si, m, side, f, leaf, sm);
    }
  }
  if constexpr (NW != kSearchWarps) return;  // the host gives the decision to a 256-thread launch
  if (!decide) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned c = atomicAdd(&st->search_done, 1u);
    last = c == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  decide_split(J, p, feats, true, &dec);
  if (threadIdx.x == 0) st->search_done = 0u;
}

// The bookkeeping of a tree's last split when it was partitioned in one pass (no histogram launch
// follows it to apply it).
__global__ void __launch_bounds__(32) k_apply_split(const JobTable jobs, Params p, int par) {
  const Job& J = jobs.job[blockIdx.z];
  JobState* st = J.st;
  if (st->stop) return;
  const SplitOutcome o = split_outcome(p, st, __ldcg(&st->pcnt[par][0]));
  post_split_writes(J, p, o, (int)threadIdx.x);
}

// Root of a tree (serial.rs:658-776 after the root sums, then :580-586 and the first
// BeforeFindBestSplit). leaf_sum[0] and root_count are already set.
__global__ void __launch_bounds__(256) k_tree_begin(const Job* __restrict__ jobs, Params p) {
  const Job& J = jobs[blockIdx.z];
  JobState* st = J.st;
  for (int i = threadIdx.x; i < p.num_leaves; i += blockDim.x) {
    J.leaf_begin[i] = 0;
    J.leaf_count[i] = i == 0 ? st->root_count : 0;
    J.leaf_buf[i] = 0;
    J.leaf_depth[i] = 0;
    J.leaf_slot[i] = -1;
    J.leaf_value[i] = 0.0;
    J.bgain[i] = -CUDART_INF;
    J.bfeat[i] = -1;
    J.bsplit[i] = (int64_t)-1 * 4294967296LL;
  }
  if (p.n_icons > 0) {  // serial.rs:660-662: every leaf's path starts empty
    uint32_t* paths = leaf_path_bits(J, p, 0);
    for (int i = threadIdx.x; i < p.num_leaves * p.path_words; i += blockDim.x) paths[i] = 0u;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    if (lane == 0) {
      st->stop = 0;
      st->tree_leaves = 1;
      st->next_free = 0;
      st->pcnt[0][0] = st->pcnt[0][1] = st->pcnt[1][0] = st->pcnt[1][1] = 0;
      const LeafSum r = J.leaf_sum[0];
      double root = leaf_output_root(p, r.sg, r.sh, r.num_data);
      st->root_output = round_to_zero(root);
      J.leaf_value[0] = st->root_output;
    }
    __syncwarp();
    before_find_best_split(J, p, st, 0, -1, lane);
  }
}

}  // namespace

void launch_search(const Job* h_jobs, int num_jobs, const Params& p, const DevFeature* feats, int clear_par,
                   bool decide, int post, cudaStream_t s) {
  const bool plain = !p.use_l1 && !p.use_max && !p.use_smooth;
  // 64-thread CTAs when every feature's slice fits in 63 bins (thread 63 holds the forward scan's
  // position -1), no feature is categorical and no CTA has to run the 256-thread decision
  const bool narrow = plain && p.search_narrow && !decide;
  const int dec = decide ? 1 : 0;
  for_job_groups(h_jobs, num_jobs, [&](const JobTable& t, int nz) {
    dim3 grid((unsigned)(2 * p.F), 1, nz);
    if (narrow) {
      const dim3 block(64);
      if (p.quant) (void)launch_kernel(k_search<true, true, 2>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
      else (void)launch_kernel(k_search<true, false, 2>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
      return;
    }
    const dim3 block(kSearchThreads);
    if (p.quant) {
      if (plain) (void)launch_kernel(k_search<true, true, 8>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
      else (void)launch_kernel(k_search<false, true, 8>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
    } else {
      if (plain) (void)launch_kernel(k_search<true, false, 8>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
      else (void)launch_kernel(k_search<false, false, 8>, grid, block, 0, s, p.pdl, t, p, feats, clear_par, dec, post);
    }
  });
}

void launch_apply_split(const Job* h_jobs, int num_jobs, const Params& p, int par, cudaStream_t s) {
  for_job_groups(h_jobs, num_jobs, [&](const JobTable& t, int nz) {
    k_apply_split<<<dim3(1, 1, nz), 32, 0, s>>>(t, p, par);
  });
}

void launch_tree_begin(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s) {
  k_tree_begin<<<dim3(1, 1, num_jobs), 256, 0, s>>>(d_jobs, p);
}

}  // namespace bk

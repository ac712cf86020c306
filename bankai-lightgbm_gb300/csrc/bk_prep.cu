// Per-tree preparation and finishing kernels of the GB300 learner:
//   - row-index initialisation (DataPartition::init / init_with, data_partition.rs:90-107);
//   - gradient discretization (GradientDiscretizer, gradient_discretizer/mod.rs:116-201) with the
//     per-tree stochastic-rounding rotation drawn on the device from a std::mt19937 state
//     (mt19937.rs:32-128), so every draw happens exactly when the reference draws;
//   - root leaf sums (serial.rs:705-775);
//   - quantized leaf renewal (serial.rs:634-655), summed sequentially in leaf row order like the
//     reference so the f64 sums round identically;
//   - score update and leaf lookup over the final partition (serial.rs:1974-1990).
#include <math_constants.h>

#include "bk_math.cuh"

namespace bk {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__global__ void k_init_rows(const Job* __restrict__ jobs, Params p, const int32_t* __restrict__ rows) {
  const Job& J = jobs[blockIdx.z];
  const int64_t cnt = J.st->root_count;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x)
    J.idx0[i] = J.st->use_rows ? rows[i] : (int32_t)i;
}

// ---- std::mt19937 on the device (one thread per job) ----
__device__ void mt_twist(uint32_t* st) {
  for (int i = 0; i < 624; ++i) {
    uint32_t y = (st[i] & 0x80000000u) | (st[(i + 1) % 624] & 0x7fffffffu);
    uint32_t nx = st[(i + 397) % 624] ^ (y >> 1);
    if (y & 1u) nx ^= 0x9908b0dfu;
    st[i] = nx;
  }
}

__device__ uint32_t mt_next(JobState* s) {
  if (s->mt_idx >= 624) {
    mt_twist(s->mt);
    s->mt_idx = 0;
  }
  uint32_t y = s->mt[s->mt_idx++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// libc++ uniform_int_distribution<int>(0, n) (mt19937.rs:109-128).
__device__ uint32_t mt_uniform_int_inclusive(JobState* s, uint32_t n) {
  uint32_t rp = n + 1u;
  if (rp == 1u) return 0u;
  if (rp == 0u) return mt_next(s);
  uint32_t w = 32u - (uint32_t)__clz(rp) - 1u;
  if (rp & (0xffffffffu >> (32u - w))) w += 1u;
  uint32_t mask = w >= 32u ? 0xffffffffu : ((1u << w) - 1u);
  for (int guard = 0; guard < 1 << 20; ++guard) {  // rejection succeeds with probability >= 1/2
    uint32_t u = mt_next(s) & mask;
    if (u < rp) return u;
  }
  return 0u;
}

__global__ void k_mt_seed(const Job* __restrict__ jobs, uint32_t seed) {
  JobState* s = jobs[blockIdx.z].st;
  s->mt[0] = seed;
  for (int i = 1; i < 624; ++i) s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->mt_idx = 624;
}

// ---- discretization ----
__global__ void k_disc_reset(const Job* __restrict__ jobs) {
  JobState* s = jobs[blockIdx.z].st;
  s->red_maxg = 0u;
  s->red_maxh = 0u;
  s->red_flags = 0u;
}

// max |g| and max h over all rows (order-free), and the refused cases (mod.rs:134-155).
__global__ void k_disc_reduce(const Job* __restrict__ jobs, Params p) {
  const Job& J = jobs[blockIdx.z];
  float mg = 0.f, mh = 0.f;
  uint32_t bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
    float g = J.g[i], h = J.h[i];
    if (!isfinite(g) || !isfinite(h) || h < 0.f) bad = 1u;
    mg = fmaxf(mg, fabsf(g));
    mh = fmaxf(mh, h);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mg = fmaxf(mg, __shfl_xor_sync(FULL, mg, o));
    mh = fmaxf(mh, __shfl_xor_sync(FULL, mh, o));
    bad |= __shfl_xor_sync(FULL, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    // non-negative floats order like their bit patterns
    atomicMax(&J.st->red_maxg, __float_as_uint(mg));
    atomicMax(&J.st->red_maxh, __float_as_uint(mh));
    if (bad) atomicOr(&J.st->red_flags, 1u);
  }
}

// One thread for all jobs, in job order: the K class trees of an iteration share one
// discretizer, so their rotation offsets are consecutive draws of one engine (held by job 0).
__global__ void k_disc_setup(const Job* __restrict__ jobs, int num_jobs, Params p) {
  JobState* eng = jobs[0].st;
  for (int j = 0; j < num_jobs; ++j) {
    JobState* s = jobs[j].st;
    float max_g = __uint_as_float(s->red_maxg), max_h = __uint_as_float(s->red_maxh);
    bool ok = s->red_flags == 0u && max_g != 0.f && (p.const_hess || max_h != 0.f);
    s->disc_ok = ok ? 1 : 0;
    if (!ok) continue;  // the reference warns and keeps the previous discretization (serial.rs:692-703)
    s->gscale = (double)max_g / (double)(p.quant_bins / 2);
    s->hscale = p.const_hess ? (double)max_h : (double)max_h / (double)p.quant_bins;
    s->inv_g = 1.0 / s->gscale;
    s->inv_h = 1.0 / s->hscale;
    if (p.stochastic) s->start_pos = mt_uniform_int_inclusive(eng, (uint32_t)p.n);
  }
}

__device__ __forceinline__ int32_t sat_i8(double v) {  // Rust `f64 as i8`
  if (isnan(v)) return 0;
  if (v >= 127.0) return 127;
  if (v <= -128.0) return -128;
  return (int32_t)trunc(v);
}

__global__ void k_discretize(const Job* __restrict__ jobs, Params p, const double* __restrict__ noise_g,
                             const double* __restrict__ noise_h) {
  const Job& J = jobs[blockIdx.z];
  const JobState* s = J.st;
  if (!s->disc_ok) return;
  const double ig = s->inv_g, ih = s->inv_h;
  const bool fused = p.fused != 0;
  const int64_t start = s->start_pos;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
    double gv = (double)J.g[i];
    int32_t gi, hi;
    if (p.stochastic) {
      int64_t pos = i + start;
      if (pos >= p.n) pos -= p.n;
      double noise = noise_g[pos];
      double sn = gv >= 0.0 ? noise : -noise;
      gi = sat_i8(madd(gv, ig, sn, fused));
      hi = p.const_hess ? 1 : sat_i8(madd((double)J.h[i], ih, noise_h[pos], fused));
    } else {
      double off = gv >= 0.0 ? 0.5 : -0.5;
      gi = sat_i8(madd(gv, ig, off, fused));
      hi = p.const_hess ? 1 : sat_i8(madd((double)J.h[i], ih, 0.5, fused));
    }
    J.packed[i] = (int16_t)((gi * 256) | (hi & 0xff));
  }
}

// ---- root sums ----
// Float path: Σg, Σh in f64 over the root rows; per-CTA partials summed in CTA order.
// Quantized path: exact integer sums; the f64 sums Σ(int · scale) are the integer sum times the
// scale whenever every partial sum is exactly representable (power-of-two bin counts and fewer
// than 2^29 units), which is then bit-identical to the reference's sequential sum; otherwise a
// single warp sums sequentially in row order like the reference.
__global__ void __launch_bounds__(256) k_root_partial(const Job* __restrict__ jobs, Params p) {
  __shared__ double sg_s[8], sh_s[8];
  __shared__ long long ig_s[8], ih_s[8];
  const Job& J = jobs[blockIdx.z];
  const int64_t cnt = J.st->root_count;
  double sg = 0.0, sh = 0.0;
  long long ig = 0, ih = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = J.idx0[k];
    if (p.quant) {
      int32_t pk = J.packed[i];
      ig += (int8_t)(pk >> 8);
      ih += pk & 0xff;
    } else {
      sg += (double)J.g[i];
      sh += (double)J.h[i];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sg += __shfl_xor_sync(FULL, sg, o);
    sh += __shfl_xor_sync(FULL, sh, o);
    ig += __shfl_xor_sync(FULL, ig, o);
    ih += __shfl_xor_sync(FULL, ih, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sg_s[warp] = sg;
    sh_s[warp] = sh;
    ig_s[warp] = ig;
    ih_s[warp] = ih;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    long long c = 0, d = 0;
    for (int w = 0; w < 8; ++w) {
      a += sg_s[w];
      b += sh_s[w];
      c += ig_s[w];
      d += ih_s[w];
    }
    J.red[2 * blockIdx.x] = a;
    J.red[2 * blockIdx.x + 1] = b;
    J.ired[2 * blockIdx.x] = c;
    J.ired[2 * blockIdx.x + 1] = d;
  }
}

__global__ void k_root_finish(const Job* __restrict__ jobs, Params p, int exact_quant_root) {
  const Job& J = jobs[blockIdx.z];
  JobState* s = J.st;
  const int lane = threadIdx.x;
  double sg = 0.0, sh = 0.0;
  int64_t ig = 0, ih = 0;
  if (lane == 0) {
    for (int b = 0; b < kRootGrid; ++b) {
      sg += J.red[2 * b];
      sh += J.red[2 * b + 1];
      ig += J.ired[2 * b];
      ih += J.ired[2 * b + 1];
    }
  }
  if (p.quant && !exact_quant_root) {
    // sequential f64 sum of int * scale in root row order (serial.rs:717-739)
    double a = 0.0, b = 0.0;
    const int64_t cnt = s->root_count;
    for (int64_t base = 0; base < cnt; base += 32) {
      int64_t k = base + lane;
      int32_t gi = 0, hi = 0;
      if (k < cnt) {
        int32_t pk = J.packed[J.idx0[k]];
        gi = (int8_t)(pk >> 8);
        hi = pk & 0xff;
      }
      int jn = (int)min((int64_t)32, cnt - base);
      for (int j = 0; j < jn; ++j) {
        int32_t g = __shfl_sync(FULL, gi, j), h = __shfl_sync(FULL, hi, j);
        if (lane == 0) {
          a += (double)g * s->gscale;
          b += (double)h * s->hscale;
        }
      }
    }
    sg = a;
    sh = b;
  } else if (p.quant) {
    sg = (double)ig * s->gscale;
    sh = (double)ih * s->hscale;
  }
  if (lane == 0) {
    LeafSum r;
    r.sg = sg;
    r.sh = sh;
    r.weight = 0.0;
    r.int_sum = p.quant ? (int64_t)((uint64_t)ig * 4294967296ull + (uint64_t)ih) : 0;
    r.num_data = (int32_t)s->root_count;
    r._pad = 0;
    J.leaf_sum[0] = r;
  }
}

// ---- leaf renewal (quantized, quant_train_renew_leaf) ----
__global__ void __launch_bounds__(32) k_renew(const Job* __restrict__ jobs, Params p) {
  const Job& J = jobs[blockIdx.z];
  const int32_t leaf = blockIdx.x;
  if (leaf >= J.st->tree_leaves) return;
  const int lane = threadIdx.x;
  const int64_t begin = J.leaf_begin[leaf], cnt = J.leaf_count[leaf];
  const int32_t* idx = leaf_idx(J, J.leaf_buf[leaf]) + begin;
  double s1 = 0.0, s2 = 0.0;
  for (int64_t base = 0; base < cnt; base += 32) {
    int64_t k = base + lane;
    float gv = 0.f, hv = 0.f;
    if (k < cnt) {
      int32_t r = idx[k];
      gv = J.g[r];
      hv = J.h[r];
    }
    int jn = (int)min((int64_t)32, cnt - base);
    for (int j = 0; j < jn; ++j) {
      float a = __shfl_sync(FULL, gv, j), b = __shfl_sync(FULL, hv, j);
      s1 += (double)a;
      s2 += (double)b;
    }
  }
  if (lane == 0) {
    double o = leaf_output(true, true, false, s1, s2, p, (int32_t)cnt, 0.0);
    J.leaf_value[leaf] = round_to_zero(o);
  }
}

// ---- score update / leaf lookup over the final partition ----
__global__ void k_add_score(const Job* __restrict__ jobs, Params p, const double* __restrict__ vals,
                            double* __restrict__ score) {
  const Job& J = jobs[blockIdx.z];
  const int32_t leaf = blockIdx.y;
  if (leaf >= J.st->tree_leaves || J.st->tree_leaves <= 1) return;
  const double v = vals[(size_t)blockIdx.z * p.num_leaves + leaf];
  const int64_t begin = J.leaf_begin[leaf], cnt = J.leaf_count[leaf];
  const int32_t* idx = leaf_idx(J, J.leaf_buf[leaf]) + begin;
  double* sc = score + (size_t)blockIdx.z * p.n;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x)
    sc[idx[k]] += v;
}

// The same update with the tree's own leaf outputs from the device, shrunk as Tree::apply_shrinkage
// does (tree.rs:446-463): score += round_to_zero(leaf_value * rate). A one-leaf tree adds nothing
// (train.rs:776-795 turns it into a constant tree instead).
__global__ void k_add_score_own(const Job* __restrict__ jobs, Params p, double rate, double* __restrict__ score) {
  const Job& J = jobs[blockIdx.z];
  const int32_t leaf = blockIdx.y;
  if (leaf >= J.st->tree_leaves || J.st->tree_leaves <= 1) return;
  double v = __dmul_rn(J.leaf_value[leaf], rate);
  if (v >= -BK_ZERO_THRESHOLD && v <= BK_ZERO_THRESHOLD) v = 0.0;
  const int64_t begin = J.leaf_begin[leaf], cnt = J.leaf_count[leaf];
  const int32_t* idx = leaf_idx(J, J.leaf_buf[leaf]) + begin;
  double* sc = score + (size_t)blockIdx.z * p.n;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x)
    sc[idx[k]] += v;
}

__global__ void k_row_leaf(const Job* __restrict__ jobs, Params p, int32_t* __restrict__ out) {
  const Job& J = jobs[blockIdx.z];
  const int32_t leaf = blockIdx.y;
  if (leaf >= J.st->tree_leaves) return;
  const int64_t begin = J.leaf_begin[leaf], cnt = J.leaf_count[leaf];
  const int32_t* idx = leaf_idx(J, J.leaf_buf[leaf]) + begin;
  int32_t* o = out + (size_t)blockIdx.z * p.n;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x)
    o[idx[k]] = leaf;
}

}  // namespace

void launch_init_rows(const Job* d_jobs, int num_jobs, const Params& p, const int32_t* rows, cudaStream_t s) {
  k_init_rows<<<dim3(1024, 1, num_jobs), 256, 0, s>>>(d_jobs, p, rows);
}

void launch_mt_seed(const Job* d_jobs, int num_jobs, uint32_t seed, cudaStream_t s) {
  (void)num_jobs;  // one engine, held by job 0
  k_mt_seed<<<1, 1, 0, s>>>(d_jobs, seed);
}

void launch_discretize(const Job* d_jobs, int num_jobs, const Params& p, const double* noise_g, const double* noise_h,
                       cudaStream_t s) {
  k_disc_reset<<<dim3(1, 1, num_jobs), 1, 0, s>>>(d_jobs);
  k_disc_reduce<<<dim3(512, 1, num_jobs), 256, 0, s>>>(d_jobs, p);
  k_disc_setup<<<1, 1, 0, s>>>(d_jobs, num_jobs, p);
  k_discretize<<<dim3(1024, 1, num_jobs), 256, 0, s>>>(d_jobs, p, noise_g, noise_h);
}

void launch_root_sums(const Job* d_jobs, int num_jobs, const Params& p, int exact_quant_root, cudaStream_t s) {
  k_root_partial<<<dim3(kRootGrid, 1, num_jobs), 256, 0, s>>>(d_jobs, p);
  k_root_finish<<<dim3(1, 1, num_jobs), 32, 0, s>>>(d_jobs, p, exact_quant_root);
}

void launch_renew(const Job* d_jobs, int num_jobs, const Params& p, cudaStream_t s) {
  k_renew<<<dim3(p.num_leaves, 1, num_jobs), 32, 0, s>>>(d_jobs, p);
}

void launch_add_score(const Job* d_jobs, int num_jobs, const Params& p, const double* leaf_vals, double* score,
                      cudaStream_t s) {
  k_add_score<<<dim3(8, p.num_leaves, num_jobs), 256, 0, s>>>(d_jobs, p, leaf_vals, score);
}

void launch_add_score_own(const Job* d_jobs, int num_jobs, const Params& p, double rate, double* score,
                          cudaStream_t s) {
  k_add_score_own<<<dim3(8, p.num_leaves, num_jobs), 256, 0, s>>>(d_jobs, p, rate, score);
}

void launch_row_leaf(const Job* d_jobs, int num_jobs, const Params& p, int32_t* out, cudaStream_t s) {
  k_row_leaf<<<dim3(8, p.num_leaves, num_jobs), 256, 0, s>>>(d_jobs, p, out);
}

}  // namespace bk

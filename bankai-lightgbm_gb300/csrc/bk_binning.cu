// Dense bin construction on the device: the O(rows x features) part of Dataset::from_dense and
// Dataset::from_dense_reference (io/dataset.rs:633-685 fill_dense, io/dataset.rs:987-1003), with
// BinMapper::value_to_bin (io/bin.rs:558-589) per value. The bin mappers themselves (upper bounds,
// missing type, most frequent bin) come from the host's BinMapper::find_bin over a row sample, as
// in the reference; this file turns a device-resident value matrix into the learner's stored-bin
// columns.
//
// Layout: the values are row-major [num_data][num_columns], f64 or f32. A CTA owns 16 used
// features and a run of 2048 rows; the flat grid runs feature groups fastest, so the CTAs that
// read the same rows' lines run side by side. A CTA keeps its features' bounds in shared memory,
// padded to 256 entries with +inf, and walks its rows in tiles of 256: the tile's values are read
// row by row (coalesced) into shared memory, then each warp bins 32 rows of ONE feature with a
// branchless 8-step search (the number of bounds below the value, which is value_to_bin's
// binary-search result for sorted bounds), and each feature's 256 stored bins leave as one
// contiguous segment of its column.
//
// GB300 issues one warp f64 instruction per 64 cycles per SM sub-partition, so no f64 arithmetic
// runs per value: the searches compare order-preserving integer keys (-0.0 folded into +0.0, as
// the f64 comparison treats them; NaN, found from the bits, never reaches the search). An f64
// value's key is built from its bits. An f32 value is compared in f32 against its bound rounded
// down to f32, which is exact: a float v satisfies v <= ub exactly when v <= the largest float
// not above ub.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "bk_common.cuh"
#include "bkgpu.h"

namespace bk {

namespace {

constexpr int kBinRows = 256;     // rows per tile
constexpr int kBinTiles = 8;      // tiles per CTA
constexpr int kBinFeatures = 16;  // used features per CTA
constexpr int kBinThreads = 256;

struct BinFeature {
  int32_t real, num_bin, missing, mfb, ub_off;
};

// Integer keys whose signed order is the order of the non-NaN values (-0.0 taken as +0.0): int64
// keys of f64 values and bounds, int32 keys of f32 values and of the bounds rounded down to f32.
// kNanKey marks a NaN of a feature whose NaN has its own bin; it is below every real key.
__device__ __forceinline__ long long order_key(long long b) {
  if ((b << 1) == 0) b = 0;  // -0.0
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ int order_key(int b) {
  if ((b << 1) == 0) b = 0;  // -0.0f
  return b ^ ((b >> 31) & 0x7fffffff);
}

template <typename T>
struct KeyOf;
template <>
struct KeyOf<double> {
  using K = long long;
  static constexpr K kNanKey = (K)0x8000000000000000ULL;
  __device__ static K bound(double ub) { return order_key(__double_as_longlong(ub)); }
  __device__ static bool nan(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
  }
  __device__ static K value(double v) { return order_key(__double_as_longlong(v)); }
};
template <>
struct KeyOf<float> {
  using K = int;
  static constexpr K kNanKey = (K)0x80000000u;
  __device__ static K bound(double ub) { return order_key(__float_as_int(__double2float_rd(ub))); }
  __device__ static bool nan(float v) { return (__float_as_int(v) & 0x7fffffff) > 0x7f800000; }
  __device__ static K value(float v) { return order_key(__float_as_int(v)); }
};

template <typename K>
struct BinSmem {
  K sk[kBinFeatures][256];           // bound keys, +inf past the searched ones
  K xs[kBinRows][kBinFeatures + 1];  // value keys; +1: a warp's 32 rows of one feature hit 32 banks
  BinFeature sf[kBinFeatures];
  uint8_t stage[kBinFeatures][kBinRows];
};

template <typename T>
__global__ void __launch_bounds__(kBinThreads)
    k_bin_dense(const T* __restrict__ X, int64_t n, int32_t ncol, const BinFeature* __restrict__ feats, int32_t F,
                const double* __restrict__ ub, uint8_t* __restrict__ out) {
  using KO = KeyOf<T>;
  using K = typename KO::K;
  extern __shared__ __align__(16) unsigned char bin_smem[];
  BinSmem<K>& S = *reinterpret_cast<BinSmem<K>*>(bin_smem);
  const int ngroups = (F + kBinFeatures - 1) / kBinFeatures;
  const int g0 = (int)(blockIdx.x % (unsigned)ngroups) * kBinFeatures;
  const int64_t chunk = blockIdx.x / (unsigned)ngroups;
  const int gf = min(kBinFeatures, F - g0);
  if (threadIdx.x < gf) S.sf[threadIdx.x] = feats[g0 + threadIdx.x];
  __syncthreads();
  const K kInf = KO::bound(CUDART_INF);
  for (int e = threadIdx.x; e < kBinFeatures * 256; e += kBinThreads) {
    const int fi = e >> 8, i = e & 255;
    K k = kInf;
    if (fi < gf) {
      const BinFeature m = S.sf[fi];
      const int rr = m.num_bin - 1 - (m.missing == 2 ? 1 : 0);  // the searched bounds
      if (i < rr) k = KO::bound(ub[m.ub_off + i]);
    }
    S.sk[fi][i] = k;
  }
  for (int tile = 0; tile < kBinTiles; ++tile) {
    const int64_t r0 = (chunk * kBinTiles + tile) * kBinRows;
    if (r0 >= n) break;  // uniform
    const int rows = (int)min((int64_t)kBinRows, n - r0);
    __syncthreads();  // the previous tile's stage is written out; sk is complete
    for (int e = threadIdx.x; e < kBinRows * kBinFeatures; e += kBinThreads) {
      const int ri = e >> 4, fi = e & (kBinFeatures - 1);
      if (ri < rows && fi < gf) {
        const BinFeature& m = S.sf[fi];
        const T v = X[(r0 + ri) * (int64_t)ncol + m.real];
        // value_to_bin's NaN: its own bin (missing NaN) or the value 0.0
        S.xs[ri][fi] = KO::nan(v) ? (m.missing == 2 ? KO::kNanKey : KO::value((T)0)) : KO::value(v);
      }
    }
    __syncthreads();
    const int ri = threadIdx.x;  // a warp: 32 rows of one feature at a time
    for (int fi = 0; fi < gf; ++fi) {
      if (ri >= rows) break;
      const BinFeature m = S.sf[fi];
      const K vk = S.xs[ri][fi];
      int32_t bin;
      if (vk == KO::kNanKey) {
        bin = m.num_bin - 1;  // the NaN bin
      } else {
        // value_to_bin (bin.rs:576-585): the first searched bound >= v, i.e. the number of
        // searched bounds below v (the bounds are sorted)
        const K* b = S.sk[fi];
        int pos = 0;
#pragma unroll
        for (int step = 128; step >= 1; step >>= 1) pos += b[pos + step - 1] < vk ? step : 0;
        bin = pos;
      }
      // fill_dense: the most frequent bin is stored as 0, the others shift past it
      S.stage[fi][ri] = (uint8_t)(bin == m.mfb ? 0 : bin + 1 - (m.mfb == 0 ? 1 : 0));
    }
    __syncthreads();
    for (int e = threadIdx.x; e < gf * kBinRows; e += kBinThreads) {
      const int fi = e >> 8, r = e & (kBinRows - 1);
      if (r < rows) out[(size_t)(g0 + fi) * (size_t)n + (size_t)(r0 + r)] = S.stage[fi][r];
    }
  }
}

// The smallest flat index (feature * n + row) whose stored bin is outside its feature's
// [0, gbins), or INT64_MAX: the reference's BinsCheck (histogram.rs:50-65) over device columns.
__global__ void __launch_bounds__(256)
    k_check_bins(const uint8_t* __restrict__ bins, int64_t n, const DevFeature* __restrict__ feats,
                 unsigned long long* first_bad) {
  const int f = blockIdx.y;
  const uint32_t gb = (uint32_t)feats[f].gbins;
  const uint8_t* col = bins + (size_t)f * (size_t)n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if ((uint32_t)col[i] >= gb) atomicMin(first_bad, (unsigned long long)((int64_t)f * n + i));
}

}  // namespace

cudaError_t check_bins_device(const uint8_t* bins, int64_t n, int32_t F, const DevFeature* d_feat,
                              int64_t* first_bad, cudaStream_t s) {
  unsigned long long* d_bad = nullptr;
  cudaError_t e = cudaMalloc(&d_bad, sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  const unsigned long long none = ~0ull;
  e = cudaMemcpyAsync(d_bad, &none, sizeof(none), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    const int gx = (int)std::min<int64_t>(ceil_div64(n, 256), 64);
    k_check_bins<<<dim3(gx, F), 256, 0, s>>>(bins, n, d_feat, d_bad);
    e = cudaGetLastError();
  }
  unsigned long long h = none;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_bad, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_bad);
  *first_bad = h == none ? INT64_MAX : (int64_t)h;
  return e;
}

}  // namespace bk

using namespace bk;

namespace {

void bin_error(const char* msg) { bk_set_last_error(msg); }

template <typename A0, typename... A>
void bin_error(const char* fmt, A0 a0, A... a) {
  char buf[256];
  snprintf(buf, sizeof(buf), fmt, a0, a...);
  bk_set_last_error(buf);
}

}  // namespace

extern "C" int bk_bin_dense_device(const void* values, int32_t value_type, int64_t num_data, int32_t num_columns,
                                   const bk_feature* features, int32_t num_features, const double* upper_bounds,
                                   const int32_t* bound_offsets, uint8_t* out, void* stream) {
  if (!values || !features || !upper_bounds || !bound_offsets || !out || num_data <= 0 || num_columns <= 0 ||
      num_features <= 0 || (value_type != 0 && value_type != 1)) {
    bin_error("bk_bin_dense_device: invalid arguments");
    return -1;
  }
  std::vector<BinFeature> hf((size_t)num_features);
  for (int f = 0; f < num_features; ++f) {
    const bk_feature& x = features[f];
    const int32_t nb = x.num_bin, off = x.most_freq_bin == 0 ? 1 : 0;
    if (x.bin_type != 0) {
      bin_error("bk_bin_dense_device: feature %d is categorical; device binning takes numerical features", f);
      return -1;
    }
    if (x.real_feature < 0 || x.real_feature >= num_columns || nb < 1 || 1 + nb - off > 256 ||
        x.missing_type < 0 || x.missing_type > 2 || x.most_freq_bin < 0 || x.most_freq_bin >= nb ||
        bound_offsets[f] < 0 || bound_offsets[f + 1] - bound_offsets[f] != nb) {
      bin_error("bk_bin_dense_device: feature %d: bad bin mapper", f);
      return -1;
    }
    hf[(size_t)f] = BinFeature{x.real_feature, nb, x.missing_type, x.most_freq_bin, bound_offsets[f]};
  }
  const size_t nub = (size_t)bound_offsets[num_features];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  BinFeature* d_f = nullptr;
  double* d_ub = nullptr;
  cudaError_t e = cudaMalloc(&d_f, sizeof(BinFeature) * hf.size());
  if (e == cudaSuccess) e = cudaMalloc(&d_ub, sizeof(double) * nub);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_f, hf.data(), sizeof(BinFeature) * hf.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ub, upper_bounds, sizeof(double) * nub, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    // one flat grid, feature groups fastest: the CTAs reading the same rows' lines run side by side
    const int64_t groups = ceil_div64(num_features, kBinFeatures);
    const int64_t blocks = groups * ceil_div64(num_data, (int64_t)kBinRows * kBinTiles);
    if (blocks > INT32_MAX) {
      cudaFree(d_f);
      cudaFree(d_ub);
      bin_error("bk_bin_dense_device: too many rows x features for one launch");
      return -1;
    }
    dim3 grid((unsigned)blocks);
    if (value_type == 0) {
      const int smem = (int)sizeof(BinSmem<long long>);
      e = cudaFuncSetAttribute(k_bin_dense<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e == cudaSuccess)
        k_bin_dense<double><<<grid, kBinThreads, smem, s>>>(static_cast<const double*>(values), num_data,
                                                            num_columns, d_f, num_features, d_ub, out);
    } else {
      const int smem = (int)sizeof(BinSmem<int>);
      e = cudaFuncSetAttribute(k_bin_dense<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e == cudaSuccess)
        k_bin_dense<float><<<grid, kBinThreads, smem, s>>>(static_cast<const float*>(values), num_data, num_columns,
                                                           d_f, num_features, d_ub, out);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_f);
  cudaFree(d_ub);
  if (e != cudaSuccess) {
    bin_error("bk_bin_dense_device: %s", cudaGetErrorString(e));
    return -1;
  }
  return 0;
}

// A row partition that allocates nothing, for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host that hands all of the GPU's memory
// to its own caching allocator (so any allocation outside it fails or fragments the budget), or a
// latency-critical path that must not take cudaMalloc's implicit device-wide synchronization in
// the middle of its stream. For them bk_partition_split_noalloc runs DataPartition::Split's stable
// partition (data_partition.rs:124-174) on buffers the caller owns; its only scratch is the fixed
// file-scope device array below, sized for at most kMaxBlocks row chunks (8 KiB), which every GPU
// that loads this library keeps until the process exits.
//
// The array is shared by all calls and keeps the last call's contents: every slot a call reads is
// written earlier in the same call, so nothing needs clearing, but calls that overlap on the GPU
// (on different streams, or from different host threads) race on it and must be serialised.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "bk_common.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr int kMaxBlocks = 1024;
constexpr int64_t kMaxChunk = int64_t(1) << 20;
constexpr int64_t kMaxRows = (int64_t)kMaxBlocks * kMaxChunk;  // 2^30 rows
constexpr int kMaxDevices = 64;

// per-chunk left counts, the total left count at [kMaxBlocks], an out-of-range-row flag at
// [kMaxBlocks + 1]
static __device__ __align__(256) int64_t g_partition_scratch[kMaxBlocks + 2];

struct RouteTable {
  uint8_t left[256];
};

__device__ __forceinline__ int64_t block_sum(int64_t v, int64_t* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  int64_t t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
  __syncthreads();
  return t;
}

// Route of one row: rows outside the bins column go right and raise the error flag.
__device__ __forceinline__ uint8_t route_row(const uint8_t* bins, int64_t bins_len, const RouteTable& route, int32_t r,
                                             int64_t* scratch) {
  if ((uint64_t)(uint32_t)r >= (uint64_t)bins_len) {
    scratch[kMaxBlocks + 1] = 1;
    return 0;
  }
  return route.left[bins[r]];
}

__global__ void __launch_bounds__(kThreads) k_na_count(const int32_t* __restrict__ rows, int64_t n, int64_t chunk,
                                                       const uint8_t* __restrict__ bins, int64_t bins_len,
                                                       RouteTable route, int64_t* __restrict__ scratch) {
  __shared__ int64_t sh[kThreads / 32];
  const int64_t r0 = min((int64_t)blockIdx.x * chunk, n), r1 = min(r0 + chunk, n);
  int64_t local = 0;
  for (int64_t i = r0 + threadIdx.x; i < r1; i += kThreads) local += route_row(bins, bins_len, route, rows[i], scratch);
  int64_t t = block_sum(local, sh);
  if (threadIdx.x == 0) scratch[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kThreads) k_na_scatter(const int32_t* __restrict__ rows, int64_t n, int64_t chunk,
                                                         const uint8_t* __restrict__ bins, int64_t bins_len,
                                                         RouteTable route, int32_t* __restrict__ out,
                                                         int64_t* __restrict__ scratch) {
  __shared__ int64_t sh[kThreads / 32];
  __shared__ int32_t wsum[kThreads / 32];
  const int64_t r0 = min((int64_t)blockIdx.x * chunk, n), r1 = min(r0 + chunk, n);
  int64_t before = 0, all = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) {
    int64_t c = scratch[b];
    all += c;
    if (b < (int)blockIdx.x) before += c;
  }
  const int64_t total_left = block_sum(all, sh);
  int64_t running = block_sum(before, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) scratch[kMaxBlocks] = total_left;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = r0; base < r1; base += kTile) {
    const int64_t e0 = base + (int64_t)threadIdx.x * kItems;
    int32_t rr[kItems];
    uint32_t flags = 0;
    int32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      rr[k] = 0;
      if (e0 + k < r1) {
        rr[k] = rows[e0 + k];
        if (route_row(bins, bins_len, route, rr[k], scratch)) {
          flags |= 1u << k;
          ++cnt;
        }
      }
    }
    // block-wide exclusive scan of the per-thread left counts (threads in row order)
    int32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t u = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += u;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int32_t wpre = 0, tile_total = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      if (w < warp) wpre += wsum[w];
      tile_total += wsum[w];
    }
    __syncthreads();
    int64_t left_before = running + wpre + (x - cnt);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int64_t e = e0 + k;
      if (e < r1) {
        if (flags & (1u << k)) out[left_before++] = rr[k];
        else out[total_left + (e - left_before)] = rr[k];
      }
    }
    running += tile_total;
  }
}

std::mutex g_setup_mutex;
int64_t* g_scratch_ptr[kMaxDevices] = {};

}  // namespace

extern "C" int bk_partition_split_noalloc(const int32_t* rows_in, int64_t num_rows, const uint8_t* bins,
                                          int64_t bins_len, const uint8_t* route, int32_t* rows_out,
                                          int64_t* num_left, void* stream) {
  if (!rows_in || !bins || !route || !rows_out || !num_left || num_rows < 0 || bins_len < 0 ||
      rows_in == rows_out) {
    bk_set_last_error("bk_partition_split_noalloc: invalid arguments");
    return -1;
  }
  if (num_rows > kMaxRows) {
    bk_set_last_error("bk_partition_split_noalloc: num_rows exceeds the fixed scratch's maximum of 2^30 rows "
                      "(1024 chunks of at most 2^20 rows)");
    return -1;
  }
  // an error left on this thread by earlier, unrelated work must not fail this call
  (void)cudaGetLastError();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    bk_set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "bk_partition_split_noalloc: device id too large");
    return -1;
  }
  int64_t* scratch = nullptr;
  {
    // once per device, with that device current: the device address of the scratch array (in
    // host code the symbol itself is only a host-side stand-in)
    std::lock_guard<std::mutex> g(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_partition_scratch);
      if (e != cudaSuccess) {
        bk_set_last_error(cudaGetErrorString(e));
        return -1;
      }
      g_scratch_ptr[dev] = static_cast<int64_t*>(ptr);
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_rows == 0) {
    *num_left = 0;
    return 0;
  }
  int blocks = (int)std::min<int64_t>(kMaxBlocks, (num_rows + kTile - 1) / kTile);
  int64_t chunk = (num_rows + blocks - 1) / blocks;
  chunk = (chunk + kTile - 1) / kTile * kTile;
  RouteTable rt;
  for (int b = 0; b < 256; ++b) rt.left[b] = route[b] ? 1 : 0;
  // the error flag must start at zero; the counts are overwritten by every call
  e = cudaMemsetAsync(scratch + kMaxBlocks + 1, 0, sizeof(int64_t), s);
  if (e != cudaSuccess) {
    bk_set_last_error(cudaGetErrorString(e));
    return -1;
  }
  k_na_count<<<blocks, kThreads, 0, s>>>(rows_in, num_rows, chunk, bins, bins_len, rt, scratch);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_na_scatter<<<blocks, kThreads, 0, s>>>(rows_in, num_rows, chunk, bins, bins_len, rt, rows_out, scratch);
    e = cudaGetLastError();
  }
  int64_t result[2] = {0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(result, scratch + kMaxBlocks, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    bk_set_last_error(cudaGetErrorString(e));
    return -1;
  }
  if (result[1]) {
    bk_set_last_error("bk_partition_split_noalloc: a row id is outside the bins column");
    return -1;
  }
  *num_left = result[0];
  return 0;
}

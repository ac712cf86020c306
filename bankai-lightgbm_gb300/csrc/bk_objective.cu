// Built-in objective gradients on the device, written into the learner's gradient buffers, and
// the training loss, so one boosting iteration (gradients, K trees, score update) stays in HBM:
//   L2         objective/regression.rs:240-248   g = (score - label) as f32, h = 1
//              weighted, regression.rs:321-329   g = ((score - label) as f32) * w, h = w
//   binary     objective/binary.rs:71-90         response = -label*s / (1 + exp(label*s*score)),
//                                                times the label weight of the row's class
//                                                (binary.rs:33-52) and the row weight
//   multiclass objective/multiclass.rs:68-90     softmax over the K class scores of a row, times
//                                                the row weight
// Operation order follows the reference. Row weights (`w`, device f32 [n], or null) and the
// binary label weights are set on the learner (bk_learner_set_objective_weights). `exp` is CUDA's double-precision exp, which can differ
// from the host libm's in the last bit, so binary / multiclass gradients may differ from a host
// computation by one f32 ulp; the learner's parity is checked on given gradients.
//
// A multiclass label outside [0, K) (or NaN) is not a class: the softmax gradient treats the row
// as belonging to no class and the loss skips the row, and both count it in `bad_label`, which the
// host turns into an error (a label is never used as an index without this check).
#include <math_constants.h>

#include "bk_common.cuh"

namespace bk {

namespace {

__global__ void k_grad_l2(const double* __restrict__ score, const float* __restrict__ label, int64_t n,
                          const float* __restrict__ w, float* __restrict__ g, float* __restrict__ h) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = (float)(score[i] - (double)label[i]);
    if (w) {
      const float wi = w[i];
      g[i] = __fmul_rn(d, wi);
      h[i] = wi;
    } else {
      g[i] = d;
      h[i] = 1.0f;
    }
  }
}

__global__ void k_grad_binary(const double* __restrict__ score, const float* __restrict__ label, int64_t n,
                              double sigmoid, const float* __restrict__ w, double lw_neg, double lw_pos,
                              float* __restrict__ g, float* __restrict__ h) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool pos = label[i] > 0.0f;
    double lab = pos ? 1.0 : -1.0;
    const double lw = pos ? lw_pos : lw_neg;
    double t = -lab * sigmoid;
    double e = exp(lab * sigmoid * score[i]);
    double response = t / (1.0 + e);
    double ar = fabs(response);
    double q = ar * (sigmoid - ar);
    if (w) {
      const double wi = (double)w[i];
      g[i] = (float)(response * lw * wi);
      h[i] = (float)(q * lw * wi);
    } else {
      g[i] = (float)(response * lw);
      h[i] = (float)(q * lw);
    }
  }
}

// The class of a multiclass label, or -1 (counted in *bad_label) when it is not in [0, K).
__device__ __forceinline__ int class_of(float lf, int K, int32_t* bad_label) {
  if (lf >= 0.0f && lf < (float)K) return (int)lf;
  atomicAdd(bad_label, 1);
  return -1;
}

__global__ void k_grad_softmax(const double* __restrict__ score, const float* __restrict__ label, int64_t n, int K,
                               const float* __restrict__ w, float* __restrict__ g, float* __restrict__ h,
                               int32_t* __restrict__ bad_label) {
  const double factor = (double)K / ((double)K - 1.0);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double rec[32];
    double wmax = score[i];
    for (int k = 1; k < K; ++k) wmax = fmax(score[(size_t)k * n + i], wmax);
    double wsum = 0.0;
    for (int k = 0; k < K; ++k) {
      rec[k] = exp(score[(size_t)k * n + i] - wmax);
      wsum += rec[k];
    }
    const int lab = class_of(label[i], K, bad_label);
    const double wi = w ? (double)w[i] : 1.0;
    for (int k = 0; k < K; ++k) {
      double p = rec[k] / wsum;
      double gi = lab == k ? p - 1.0 : p;
      double hi = factor * p;
      hi = hi * (1.0 - p);
      g[(size_t)k * n + i] = (float)(w ? gi * wi : gi);
      h[(size_t)k * n + i] = (float)(w ? hi * wi : hi);
    }
  }
}

// Per-CTA partial losses (mean squared error / log loss / multiclass log loss).
__global__ void k_loss(int kind, const double* __restrict__ score, const float* __restrict__ label, int64_t n, int K,
                       double* __restrict__ partial, int32_t* __restrict__ bad_label) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (kind == 0) {
      double d = score[i] - (double)label[i];
      acc += d * d;
    } else if (kind == 1) {
      double p = 1.0 / (1.0 + exp(-score[i]));
      p = fmin(fmax(p, 1e-15), 1.0 - 1e-15);
      acc += label[i] > 0.0f ? -log(p) : -log(1.0 - p);
    } else {
      double wmax = score[i];
      for (int k = 1; k < K; ++k) wmax = fmax(score[(size_t)k * n + i], wmax);
      double wsum = 0.0;
      for (int k = 0; k < K; ++k) wsum += exp(score[(size_t)k * n + i] - wmax);
      const int lab = class_of(label[i], K, bad_label);
      if (lab >= 0) acc += -(score[(size_t)lab * n + i] - wmax - log(wsum));
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    partial[blockIdx.x] = s;
  }
}

}  // namespace

cudaError_t objective_gradients(int kind, const double* score, const float* label, int64_t n, int K, double sigmoid,
                                const ObjectiveWeights& ow, float* g, float* h, int32_t* bad_label, cudaStream_t s) {
  const int grid = 1024, threads = 256;
  if (kind == 0) k_grad_l2<<<grid, threads, 0, s>>>(score, label, n, ow.row, g, h);
  else if (kind == 1)
    k_grad_binary<<<grid, threads, 0, s>>>(score, label, n, sigmoid, ow.row, ow.label_neg, ow.label_pos, g, h);
  else k_grad_softmax<<<grid, threads, 0, s>>>(score, label, n, K, ow.row, g, h, bad_label);
  return cudaGetLastError();
}

cudaError_t objective_loss(int kind, const double* score, const float* label, int64_t n, int K, double* partial,
                           int grid, int32_t* bad_label, cudaStream_t s) {
  k_loss<<<grid, 256, 0, s>>>(kind, score, label, n, K, partial, bad_label);
  return cudaGetLastError();
}

}  // namespace bk

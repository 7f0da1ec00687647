// mlp.cu -- the learned grid pruner's network: forward, loss gradient and Adam kernels.
//
// A fixed multilayer perceptron maps an atom's environment features to the predicted log10 of its
// quadrature error at each candidate grid level:
//   h1 = tanh(x W1 + b1),  h2 = tanh(h1 W2 + b2),  y = h2 W3 + b3,
// with kIn = 16 inputs, two hidden layers of kHid = 64 and kOut = 16 outputs (unused outputs are
// masked out of the loss).  Parameters are one float buffer: W1 [kIn][kHid], b1, W2 [kHid][kHid],
// b2, W3 [kHid][kOut], b3.  The loss is the masked mean squared error
//   L = inv_count * sum_s sum_k mask[s][k] (y[s][k] - t[s][k])^2.
// One thread handles one sample in the forward / delta kernels (the weights sit in shared memory
// and every thread reads the same address, a broadcast); the parameter gradient is one thread per
// parameter summing over the samples in a fixed order, so training is deterministic.
#include <cuda_runtime.h>

#include "../../include/calchem_xc.h"

namespace {

constexpr int kIn = 16, kHid = 64, kOut = 16;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kHid;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid * kOut;
constexpr int kParams = kOffB3 + kOut;
constexpr int kWork = 2 * kHid + 2 * kHid + kOut;  // per sample: h1, h2, d1, d2, d3
constexpr int kThreads = 128;

__device__ __forceinline__ void load_params(const float* __restrict__ p, float* s) {
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) s[i] = p[i];
  __syncthreads();
}

// Forward pass of one sample: h1, h2 and y in registers.
__device__ __forceinline__ void forward(const float* s, const float* x, float* h1, float* h2, float* y) {
#pragma unroll
  for (int j = 0; j < kHid; ++j) h1[j] = s[kOffB1 + j];
#pragma unroll
  for (int i = 0; i < kIn; ++i) {
    const float xi = x[i];
#pragma unroll
    for (int j = 0; j < kHid; ++j) h1[j] = fmaf(xi, s[kOffW1 + i * kHid + j], h1[j]);
  }
#pragma unroll
  for (int j = 0; j < kHid; ++j) h1[j] = tanhf(h1[j]);
#pragma unroll
  for (int j = 0; j < kHid; ++j) h2[j] = s[kOffB2 + j];
#pragma unroll
  for (int i = 0; i < kHid; ++i) {
    const float hi = h1[i];
#pragma unroll
    for (int j = 0; j < kHid; ++j) h2[j] = fmaf(hi, s[kOffW2 + i * kHid + j], h2[j]);
  }
#pragma unroll
  for (int j = 0; j < kHid; ++j) h2[j] = tanhf(h2[j]);
#pragma unroll
  for (int k = 0; k < kOut; ++k) y[k] = s[kOffB3 + k];
#pragma unroll
  for (int i = 0; i < kHid; ++i) {
    const float hi = h2[i];
#pragma unroll
    for (int k = 0; k < kOut; ++k) y[k] = fmaf(hi, s[kOffW3 + i * kOut + k], y[k]);
  }
}

__global__ void __launch_bounds__(kThreads) mlp_forward_kernel(const float* __restrict__ p, const float* __restrict__ x,
                                                               int n, float* __restrict__ y) {
  __shared__ float s[kParams];
  load_params(p, s);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float xi[kIn], h1[kHid], h2[kHid], yo[kOut];
#pragma unroll
  for (int k = 0; k < kIn; ++k) xi[k] = x[(size_t)i * kIn + k];
  forward(s, xi, h1, h2, yo);
#pragma unroll
  for (int k = 0; k < kOut; ++k) y[(size_t)i * kOut + k] = yo[k];
}

// Per-sample activations and deltas (back-propagated dL/d(pre-activation)) into work[i][kWork]
// (h1, h2, d1, d2, d3; the row doubles as the thread's scratch), per-sample loss into loss_part[i].
__global__ void __launch_bounds__(kThreads) mlp_delta_kernel(const float* __restrict__ p, const float* __restrict__ x,
                                                             const float* __restrict__ t, const float* __restrict__ mask,
                                                             int n, float inv_count, float* __restrict__ work,
                                                             float* __restrict__ loss_part) {
  __shared__ float s[kParams];
  load_params(p, s);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* w = work + (size_t)i * kWork;
  float* h1 = w;
  float* h2 = w + kHid;
  float* d1 = w + 2 * kHid;
  float* d2 = w + 3 * kHid;
  float* d3 = w + 4 * kHid;
  float xi[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) xi[k] = x[(size_t)i * kIn + k];
#pragma unroll 4
  for (int j = 0; j < kHid; ++j) {
    float a = s[kOffB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) a = fmaf(xi[k], s[kOffW1 + k * kHid + j], a);
    h1[j] = tanhf(a);
  }
#pragma unroll 2
  for (int j = 0; j < kHid; ++j) {
    float a = s[kOffB2 + j];
#pragma unroll 8
    for (int q = 0; q < kHid; ++q) a = fmaf(h1[q], s[kOffW2 + q * kHid + j], a);
    h2[j] = tanhf(a);
  }
  float loss = 0.f;
#pragma unroll 2
  for (int k = 0; k < kOut; ++k) {
    float a = s[kOffB3 + k];
#pragma unroll 8
    for (int q = 0; q < kHid; ++q) a = fmaf(h2[q], s[kOffW3 + q * kOut + k], a);
    const float mk = mask[(size_t)i * kOut + k];
    const float r = a - t[(size_t)i * kOut + k];
    d3[k] = 2.f * mk * r * inv_count;
    loss = fmaf(mk * r, r, loss);
  }
  loss_part[i] = loss * inv_count;
#pragma unroll 2
  for (int j = 0; j < kHid; ++j) {  // d2 = (W3 d3) * (1 - h2^2)
    float a = 0.f;
#pragma unroll
    for (int k = 0; k < kOut; ++k) a = fmaf(s[kOffW3 + j * kOut + k], d3[k], a);
    d2[j] = a * (1.f - h2[j] * h2[j]);
  }
#pragma unroll 2
  for (int j = 0; j < kHid; ++j) {  // d1 = (W2 d2) * (1 - h1^2)
    float a = 0.f;
#pragma unroll 8
    for (int q = 0; q < kHid; ++q) a = fmaf(s[kOffW2 + j * kHid + q], d2[q], a);
    d1[j] = a * (1.f - h1[j] * h1[j]);
  }
}

// One thread per parameter: dL/dparam = sum over samples (fixed order) of input x delta.
__global__ void __launch_bounds__(256) mlp_grad_kernel(const float* __restrict__ x, const float* __restrict__ work,
                                                       int n, float* __restrict__ grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kParams) return;
  const float* xin = nullptr;  // left factor: x, h1 or h2 (stride), or none for a bias
  size_t lstride = 0;
  int li = 0, dcol = 0;
  bool bias = false;
  if (q < kOffB1) {
    li = q / kHid; dcol = 2 * kHid + q % kHid; xin = x; lstride = kIn;
  } else if (q < kOffW2) {
    bias = true; dcol = 2 * kHid + (q - kOffB1);
  } else if (q < kOffB2) {
    const int r = q - kOffW2;
    li = r / kHid; dcol = 3 * kHid + r % kHid; xin = work; lstride = kWork;
  } else if (q < kOffW3) {
    bias = true; dcol = 3 * kHid + (q - kOffB2);
  } else if (q < kOffB3) {
    const int r = q - kOffW3;
    li = kHid + r / kOut; dcol = 4 * kHid + r % kOut; xin = work; lstride = kWork;
  } else {
    bias = true; dcol = 4 * kHid + (q - kOffB3);
  }
  float acc = 0.f;
  for (int s = 0; s < n; ++s) {
    const float d = work[(size_t)s * kWork + dcol];
    acc = bias ? acc + d : fmaf(xin[(size_t)s * lstride + li], d, acc);
  }
  grad[q] = acc;
}

__global__ void __launch_bounds__(256) sum_kernel(const float* __restrict__ v, int n, float* __restrict__ out) {
  __shared__ float r[256];
  float a = 0.f;
  for (int i = threadIdx.x; i < n; i += 256) a += v[i];
  r[threadIdx.x] = a;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) r[threadIdx.x] += r[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = r[0];
}

__global__ void __launch_bounds__(256) adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                                                   float* __restrict__ m, float* __restrict__ v, int n, float lr,
                                                   float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace

extern "C" {

int calchem_mlp_shape(int* n_in, int* n_hidden, int* n_out, int* n_params, int* work_per_sample) {
  if (!n_in || !n_hidden || !n_out || !n_params || !work_per_sample) return -1;
  *n_in = kIn;
  *n_hidden = kHid;
  *n_out = kOut;
  *n_params = kParams;
  *work_per_sample = kWork;
  return 0;
}

int calchem_mlp_forward(const float* d_params, const float* d_x, int n, float* d_y, void* stream) {
  if (!d_params || !d_x || !d_y || n <= 0) return -1;
  mlp_forward_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, (cudaStream_t)stream>>>(d_params, d_x, n, d_y);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

int calchem_mlp_loss_grad(const float* d_params, const float* d_x, const float* d_t, const float* d_mask, int n,
                          float inv_count, float* d_work, float* d_loss_part, float* d_grad, float* d_loss,
                          void* stream) {
  if (!d_params || !d_x || !d_t || !d_mask || !d_work || !d_loss_part || !d_grad || !d_loss || n <= 0 ||
      !(inv_count > 0.f))
    return -1;
  const cudaStream_t st = (cudaStream_t)stream;
  mlp_delta_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(d_params, d_x, d_t, d_mask, n, inv_count,
                                                                       d_work, d_loss_part);
  mlp_grad_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(d_x, d_work, n, d_grad);
  sum_kernel<<<1, 256, 0, st>>>(d_loss_part, n, d_loss);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

int calchem_mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, int n_params, int step, float lr,
                     float beta1, float beta2, float eps, void* stream) {
  if (!d_params || !d_grad || !d_m || !d_v || n_params != kParams || step < 1 || !(lr > 0.f)) return -1;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<(n_params + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_params, d_grad, d_m, d_v, n_params, lr,
                                                                        beta1, beta2, eps, c1, c2);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

}  // extern "C"

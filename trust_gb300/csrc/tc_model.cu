// tc_model.cu — the per-vertex cost model of the learned schedule.
//
// A small MLP (8 fp32 features -> 32 -> 32 -> 1, ReLU) predicts log2 of the clock64 cycles a
// vertex costs the counting kernel.  It is trained here, on the GPU, by hand-written forward,
// backward and Adam kernels on the per-vertex cycles the counting kernel records
// (trust_tc_opts.record_cycles); its inference runs inside the scheduling pass of the learned
// schedule (sched_kernel in tc_split.cu).  The reference has no counterpart: its schedule is the fixed
// USE_CTA / USE_WARP split (Without-graph-partition/TC.cu:19-20, :632), which stays the fallback.
//
// Parameter layout (TC_MODEL_FLOATS floats): feature mean[8], feature inverse scale[8],
// W1[32][8], b1[32], W2[32][32], b2[32], w3[32], b3, target mean, target scale.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "tc_internal.h"
#include "tc_model.h"

namespace tc {

// ---- one sample, forward and backward, in registers ----------------------------------------
__device__ __forceinline__ float mlp_forward(const float *__restrict__ P, const float *x_raw, float *h1, float *h2) {
  float x[TC_FEATURES];
#pragma unroll
  for (int i = 0; i < TC_FEATURES; ++i) x[i] = (x_raw[i] - P[TC_OFF_MEAN + i]) * P[TC_OFF_ISCALE + i];
#pragma unroll 4
  for (int j = 0; j < TC_HIDDEN; ++j) {
    float a = P[TC_OFF_B1 + j];
#pragma unroll
    for (int i = 0; i < TC_FEATURES; ++i) a += P[TC_OFF_W1 + j * TC_FEATURES + i] * x[i];
    h1[j] = a > 0.f ? a : 0.f;
  }
  float y = P[TC_OFF_B3];
  for (int j = 0; j < TC_HIDDEN; ++j) {
    float a = P[TC_OFF_B2 + j];
#pragma unroll 8
    for (int i = 0; i < TC_HIDDEN; ++i) a += P[TC_OFF_W2 + j * TC_HIDDEN + i] * h1[i];
    h2[j] = a > 0.f ? a : 0.f;
    y += P[TC_OFF_W3 + j] * h2[j];
  }
  return y;  // normalised target units
}

__device__ float tc_model_eval(const float *__restrict__ P, const float *x_raw) {
  float h1[TC_HIDDEN], h2[TC_HIDDEN];
  const float y = mlp_forward(P, x_raw, h1, h2);
  return y * P[TC_OFF_YSCALE] + P[TC_OFF_YMEAN];
}

// Mean-squared error gradient of a batch, accumulated into G (TC_MODEL_FLOATS floats, the
// normalisation slots stay zero).  Parameters are staged in shared memory; each thread runs one
// sample; per-thread gradients are reduced over the warp with shuffles, then one atomic per
// warp and parameter.
__global__ void mlp_grad_kernel(const float *__restrict__ Pg, const float *__restrict__ X,
                                const float *__restrict__ Y, int64_t n, float *__restrict__ G, float *loss) {
  __shared__ float P[TC_MODEL_FLOATS];
  for (int i = threadIdx.x; i < TC_MODEL_FLOATS; i += blockDim.x) P[i] = Pg[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = idx < n;
  float x[TC_FEATURES], h1[TC_HIDDEN], h2[TC_HIDDEN];
  float xr[TC_FEATURES];
#pragma unroll
  for (int i = 0; i < TC_FEATURES; ++i) xr[i] = live ? X[idx * TC_FEATURES + i] : 0.f;
#pragma unroll
  for (int i = 0; i < TC_FEATURES; ++i) x[i] = (xr[i] - P[TC_OFF_MEAN + i]) * P[TC_OFF_ISCALE + i];
  const float y = mlp_forward(P, xr, h1, h2);
  const float t = live ? (Y[idx] - P[TC_OFF_YMEAN]) / P[TC_OFF_YSCALE] : y;
  const float dy = live ? 2.f * (y - t) / (float)n : 0.f;  // d(mean sq err)/dy
  float l = live ? (y - t) * (y - t) / (float)n : 0.f;
  // layer 3
  auto acc = [&](int off, float g) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) g += __shfl_xor_sync(TC_FULL_MASK, g, o);
    if (lane == 0 && g != 0.f) atomicAdd(G + off, g);
  };
  acc(TC_OFF_B3, dy);
  float dh2[TC_HIDDEN];
  for (int j = 0; j < TC_HIDDEN; ++j) {
    acc(TC_OFF_W3 + j, dy * h2[j]);
    dh2[j] = h2[j] > 0.f ? dy * P[TC_OFF_W3 + j] : 0.f;  // through ReLU
  }
  // layer 2
  float dh1[TC_HIDDEN];
  for (int i = 0; i < TC_HIDDEN; ++i) dh1[i] = 0.f;
  for (int j = 0; j < TC_HIDDEN; ++j) {
    acc(TC_OFF_B2 + j, dh2[j]);
    for (int i = 0; i < TC_HIDDEN; ++i) {
      acc(TC_OFF_W2 + j * TC_HIDDEN + i, dh2[j] * h1[i]);
      dh1[i] += dh2[j] * P[TC_OFF_W2 + j * TC_HIDDEN + i];
    }
  }
  // layer 1
  for (int j = 0; j < TC_HIDDEN; ++j) {
    const float g = h1[j] > 0.f ? dh1[j] : 0.f;
    acc(TC_OFF_B1 + j, g);
#pragma unroll
    for (int i = 0; i < TC_FEATURES; ++i) acc(TC_OFF_W1 + j * TC_FEATURES + i, g * x[i]);
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) l += __shfl_xor_sync(TC_FULL_MASK, l, o);
  if (lane == 0 && loss) atomicAdd(loss, l);
}

// Adam (Kingma & Ba 2015) over the trainable slots [TC_OFF_W1, TC_OFF_YMEAN).
__global__ void adam_kernel(float *P, const float *G, float *M, float *V, int step, float lr, float b1, float b2,
                            float eps) {
  const int i = TC_OFF_W1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= TC_OFF_YMEAN) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float mh = m / (1.f - powf(b1, (float)step));
  const float vh = v / (1.f - powf(b2, (float)step));
  P[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void predict_kernel(const float *__restrict__ Pg, const float *__restrict__ X, int64_t n,
                               float *__restrict__ out) {
  __shared__ float P[TC_MODEL_FLOATS];
  for (int i = threadIdx.x; i < TC_MODEL_FLOATS; i += blockDim.x) P[i] = Pg[i];
  __syncthreads();
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) out[idx] = tc_model_eval(P, X + idx * TC_FEATURES);
}

// deterministic initialisation (He-style uniform) from a counter-based stream
static float init_uniform(uint64_t seed, int i) {
  uint64_t x = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)i * 0xBF58476D1CE4E5B9ULL;
  x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL; x ^= x >> 27; x *= 0x94d049bb133111ebULL; x ^= x >> 31;
  return (float)((double)(x >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
}

}  // namespace tc

using namespace tc;

extern "C" {

int trust_tc_model_floats(void) { return TC_MODEL_FLOATS; }

// The model compiled into the library, written by trust_gb300/model_train.py after training on
// the GPU (tc_model_default.inc holds TC_MODEL_FLOATS floats, or nothing before the first run).
static const float k_default_model[] = {
#include "tc_model_default.inc"
};

int trust_tc_model_default(float *model) {
  if (!model) return TRUST_TC_E_ARG;
  if (sizeof(k_default_model) / sizeof(float) != (size_t)TC_MODEL_FLOATS) return TRUST_TC_E_UNSUPPORTED;
  memcpy(model, k_default_model, sizeof(float) * TC_MODEL_FLOATS);
  return TRUST_TC_OK;
}

int trust_tc_model_init(float *model, uint64_t seed) {
  if (!model) return TRUST_TC_E_ARG;
  for (int i = 0; i < TC_MODEL_FLOATS; ++i) model[i] = 0.f;
  for (int i = 0; i < TC_FEATURES; ++i) model[TC_OFF_ISCALE + i] = 1.f;
  const float s1 = sqrtf(6.f / TC_FEATURES), s2 = sqrtf(6.f / TC_HIDDEN);
  for (int i = 0; i < TC_HIDDEN * TC_FEATURES; ++i) model[TC_OFF_W1 + i] = s1 * init_uniform(seed, i);
  for (int i = 0; i < TC_HIDDEN * TC_HIDDEN; ++i) model[TC_OFF_W2 + i] = s2 * init_uniform(seed + 1, i);
  for (int i = 0; i < TC_HIDDEN; ++i) model[TC_OFF_W3 + i] = s2 * init_uniform(seed + 2, i);
  model[TC_OFF_YSCALE] = 1.f;
  return TRUST_TC_OK;
}

// Gradient of the mean squared error over (X, Y) (device arrays, N x 8 and N) at `model` (host),
// written to `grad` (host, TC_MODEL_FLOATS).  Also returns the loss.
int trust_tc_model_grad(const float *d_x, const float *d_y, int64_t n, const float *model, float *grad, float *loss) {
  if (!d_x || !d_y || n <= 0 || !model || !grad) return TRUST_TC_E_ARG;
  float *dP = nullptr, *dG = nullptr;
  cudaError_t e = cudaMalloc(&dP, sizeof(float) * (TC_MODEL_FLOATS * 2 + 1));
  if (e != cudaSuccess) return cuda_status(e);
  dG = dP + TC_MODEL_FLOATS;
  float *dL = dG + TC_MODEL_FLOATS;
  e = cudaMemcpy(dP, model, sizeof(float) * TC_MODEL_FLOATS, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dG, 0, sizeof(float) * (TC_MODEL_FLOATS + 1));
  if (e == cudaSuccess) {
    mlp_grad_kernel<<<(unsigned)((n + 127) / 128), 128>>>(dP, d_x, d_y, n, dG, dL);
    TC_NOTE_LAUNCH();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(grad, dG, sizeof(float) * TC_MODEL_FLOATS, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss) e = cudaMemcpy(loss, dL, sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dP);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

// Train `model` (host, in/out) on device arrays X (N x 8 raw features) and Y (N log2 cycles):
// feature / target normalisation from the data, then `epochs` passes of mini-batch Adam.
// Writes the final full-data loss (normalised units) to *loss.
int trust_tc_model_train(const float *d_x, const float *d_y, int64_t n, int epochs, int batch, float lr,
                         float *model, float *loss) {
  if (!d_x || !d_y || n <= 0 || epochs < 0 || batch <= 0 || !model) return TRUST_TC_E_ARG;
  // normalisation statistics on the host (N x 8 floats copied once)
  std::vector<float> hx((size_t)n * TC_FEATURES), hy((size_t)n);
  TC_CUDA_TRY(cudaMemcpy(hx.data(), d_x, sizeof(float) * hx.size(), cudaMemcpyDeviceToHost));
  TC_CUDA_TRY(cudaMemcpy(hy.data(), d_y, sizeof(float) * hy.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < TC_FEATURES; ++i) {
    double s = 0, s2 = 0;
    for (int64_t k = 0; k < n; ++k) {
      const double v = hx[(size_t)k * TC_FEATURES + i];
      s += v;
      s2 += v * v;
    }
    const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-8);
    model[TC_OFF_MEAN + i] = (float)mu;
    model[TC_OFF_ISCALE + i] = (float)(1.0 / sqrt(var));
  }
  {
    double s = 0, s2 = 0;
    for (int64_t k = 0; k < n; ++k) {
      s += hy[(size_t)k];
      s2 += (double)hy[(size_t)k] * hy[(size_t)k];
    }
    const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-8);
    model[TC_OFF_YMEAN] = (float)mu;
    model[TC_OFF_YSCALE] = (float)sqrt(var);
  }
  float *buf = nullptr;
  const size_t nf = TC_MODEL_FLOATS;
  TC_CUDA_TRY(cudaMalloc(&buf, sizeof(float) * (4 * nf + 1)));
  float *dP = buf, *dG = buf + nf, *dM = buf + 2 * nf, *dV = buf + 3 * nf, *dL = buf + 4 * nf;
  cudaError_t e = cudaMemcpy(dP, model, sizeof(float) * nf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(dM, 0, sizeof(float) * 2 * nf);
  int step = 0;
  for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
    for (int64_t off = 0; off < n && e == cudaSuccess; off += batch) {
      const int64_t cnt = std::min<int64_t>(batch, n - off);
      e = cudaMemsetAsync(dG, 0, sizeof(float) * nf);
      if (e != cudaSuccess) break;
      mlp_grad_kernel<<<(unsigned)((cnt + 127) / 128), 128>>>(dP, d_x + off * TC_FEATURES, d_y + off, cnt, dG, nullptr);
      TC_NOTE_LAUNCH();
      adam_kernel<<<(TC_MODEL_FLOATS + 255) / 256, 256>>>(dP, dG, dM, dV, ++step, lr, 0.9f, 0.999f, 1e-8f);
      TC_NOTE_LAUNCH();
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaMemset(dG, 0, sizeof(float) * (nf + 1));
  if (e == cudaSuccess) {
    mlp_grad_kernel<<<(unsigned)((n + 127) / 128), 128>>>(dP, d_x, d_y, n, dG, dL);
    TC_NOTE_LAUNCH();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(model, dP, sizeof(float) * nf, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss) e = cudaMemcpy(loss, dL, sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(buf);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

// Predicted log2 cycles for N feature rows (device arrays).
int trust_tc_model_predict(const float *d_x, int64_t n, const float *model, float *d_out) {
  if (!d_x || n < 0 || !model || (n && !d_out)) return TRUST_TC_E_ARG;
  if (n == 0) return TRUST_TC_OK;
  float *dP = nullptr;
  TC_CUDA_TRY(cudaMalloc(&dP, sizeof(float) * TC_MODEL_FLOATS));
  cudaError_t e = cudaMemcpy(dP, model, sizeof(float) * TC_MODEL_FLOATS, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    predict_kernel<<<(unsigned)((n + 127) / 128), 128>>>(dP, d_x, n, d_out);
    TC_NOTE_LAUNCH();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(dP);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

}  // extern "C"

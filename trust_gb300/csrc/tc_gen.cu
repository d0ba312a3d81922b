// tc_gen.cu — deterministic synthetic graphs on the GPU.
//
// The reference downloads SNAP / LAW graphs (Dataset/Cit-Patents/get+preprocess.sh:1,
// Preprocess/speedupIO/get.sh:1-7); there is no network here, so configurations are generated.
// Every pair i draws from a counter-based stream (splitmix64 finaliser of key + (64 i + j) * phi),
// so the output does not depend on the launch shape and matches the CPU twins bit for bit.
// All sampling is integer arithmetic on the drawn words; the only floating point is the
// Chung-Lu cumulative table, computed once on the host.
#include <math.h>

#include <algorithm>
#include <vector>

#include "tc_internal.h"

namespace tc {

typedef unsigned long long u64;

__host__ __device__ __forceinline__ u64 mix64(u64 x) {  // splitmix64 finaliser (Steele, Lea, Flood 2014)
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}
__host__ __device__ __forceinline__ u64 draw(u64 key, u64 i, u64 j) {
  return mix64(key + (i * 64 + j) * 0x9E3779B97F4A7C15ULL);
}
static u64 gen_key(u64 seed) { return mix64(seed ^ 0x243F6A8885A308D3ULL); }

__global__ void rmat_kernel(int scale, int64_t np, unsigned ta, unsigned tab, unsigned tabc, u64 key, int32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      unsigned r = (unsigned)(draw(key, (u64)i, (u64)l) >> 32);
      unsigned ub = r >= tab, vb = (r >= ta && r < tab) || r >= tabc;
      u = (u << 1) | ub;
      v = (v << 1) | vb;
    }
    reinterpret_cast<int2 *>(out)[i] = make_int2((int)u, (int)v);
  }
}

__device__ __forceinline__ int sample_cdf(const u64 *__restrict__ cdf, int64_t n, u64 r) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (cdf[mid] > r) hi = mid; else lo = mid + 1;
  }
  return (int)lo;
}

__global__ void weighted_kernel(const u64 *__restrict__ cdf, int64_t n, int64_t np, u64 key, int32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
    int u = sample_cdf(cdf, n, draw(key, (u64)i, 0) >> 1);
    int v = sample_cdf(cdf, n, draw(key, (u64)i, 1) >> 1);
    reinterpret_cast<int2 *>(out)[i] = make_int2(u, v);
  }
}

__global__ void er_kernel(int64_t n, int64_t np, u64 key, int32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
    int u = (int)(((draw(key, (u64)i, 0) >> 32) * (u64)n) >> 32);
    int v = (int)(((draw(key, (u64)i, 1) >> 32) * (u64)n) >> 32);
    reinterpret_cast<int2 *>(out)[i] = make_int2(u, v);
  }
}

// Barabasi-Albert preferential attachment with d edges per vertex, in the endpoint-copy form of
// Batagelj & Brandes (2005), "Efficient generation of large random networks", made parallel as
// in Sanders & Schulz (2016), "Scalable generation of scale-free graphs": endpoint position 2e is
// the source of edge e (vertex e / d), position 2e + 1 its target.  Vertex 0's d edges are self
// loops (the seed graph).  Edge e of vertex v >= 1 draws a position r uniformly among the 2 v d
// endpoints of earlier vertices' edges: an even r is the source (r/2)/d, an odd r is the target
// of edge (r-1)/2, found the same way.  The chain strictly decreases (expected length 2), so
// every target is a pure function of (seed, e) and any launch shape gives the same pairs.
__host__ __device__ __forceinline__ u64 mulhi64(u64 a, u64 b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ __forceinline__ u64 ba_target(u64 key, u64 e, u64 d) {
  for (;;) {
    const u64 v = e / d;
    if (v == 0) return 0;
    const u64 r = mulhi64(draw(key, e, 0), 2 * v * d);
    if ((r & 1) == 0) return (r >> 1) / d;
    e = r >> 1;
  }
}

__global__ void ba_kernel(int64_t np, int d, u64 key, int32_t *out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < np; e += (int64_t)gridDim.x * blockDim.x)
    reinterpret_cast<int2 *>(out)[e] = make_int2((int)(e / d), (int)ba_target(key, (u64)e, (u64)d));
}

static int gen_grid(int64_t np) { return (int)std::max<int64_t>(1, std::min<int64_t>((np + 255) / 256, 152 * 64)); }

}  // namespace tc

using namespace tc;

extern "C" {

// Chung-Lu cumulative table: w_i = w_max * (1 + i/i0)^(-1/(gamma-1)); i0 by bisection on the
// integral approximation of sum w = 2 * target_edges; cdf[i] = floor(2^63 * prefix_i / total).
double trust_tc_chung_lu_table(int64_t n, double gamma, double w_max, int64_t target_edges, uint64_t *cdf) {
  double alpha = 1.0 / (gamma - 1.0);
  double want = 2.0 * (double)target_edges;
  double lo = log(1e-3), hi = log(1e12);
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi), i0 = exp(mid), s;
    if (fabs(alpha - 1.0) < 1e-12) s = w_max * i0 * log(1.0 + (double)n / i0);
    else s = w_max * i0 / (1.0 - alpha) * (pow(1.0 + (double)n / i0, 1.0 - alpha) - 1.0);
    if (s < want) lo = mid; else hi = mid;
  }
  double i0 = exp(0.5 * (lo + hi));
  double total = 0.0;
  for (int64_t i = 0; i < n; ++i) total += w_max * pow(1.0 + (double)i / i0, -alpha);
  double run = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    run += w_max * pow(1.0 + (double)i / i0, -alpha);
    double f = run / total;
    if (f > 1.0) f = 1.0;
    cdf[i] = (uint64_t)(f * 9223372036854775808.0);
  }
  if (n > 0) cdf[n - 1] = (uint64_t)1 << 63;
  return i0;
}

int trust_tc_gen_rmat_device(trust_tc_ctx *ctx, int scale, int64_t npairs, double a, double b, double c,
                             uint64_t seed, int32_t *d_pairs) {
  if (scale < 1 || scale > 31 || npairs < 0 || (npairs && !d_pairs)) return TRUST_TC_E_ARG;
  if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return TRUST_TC_E_ARG;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  const double s32 = 4294967296.0;
  unsigned ta = (unsigned)std::min(a * s32, s32 - 1), tab = (unsigned)std::min((a + b) * s32, s32 - 1),
           tabc = (unsigned)std::min((a + b + c) * s32, s32 - 1);
  if (npairs) {
    rmat_kernel<<<gen_grid(npairs), 256>>>(scale, npairs, ta, tab, tabc, gen_key(seed), d_pairs);
    TC_NOTE_LAUNCH();
  }
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaDeviceSynchronize());
  return TRUST_TC_OK;
}

int trust_tc_gen_chung_lu_device(trust_tc_ctx *ctx, int64_t n, double gamma, double w_max, int64_t target_edges,
                                 int64_t npairs, uint64_t seed, int32_t *d_pairs) {
  if (n < 1 || n >= ((int64_t)1 << 31) || gamma <= 1.0 || w_max <= 0 || target_edges < 1 || npairs < 0 ||
      (npairs && !d_pairs))
    return TRUST_TC_E_ARG;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  std::vector<uint64_t> cdf((size_t)n);
  trust_tc_chung_lu_table(n, gamma, w_max, target_edges, cdf.data());
  uint64_t *d_cdf = nullptr;
  TC_CUDA_TRY(cudaMalloc(&d_cdf, sizeof(uint64_t) * (size_t)n));
  cudaError_t e = cudaMemcpy(d_cdf, cdf.data(), sizeof(uint64_t) * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && npairs) {
    weighted_kernel<<<gen_grid(npairs), 256>>>((const u64 *)d_cdf, n, npairs, gen_key(seed), d_pairs);
    TC_NOTE_LAUNCH();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(d_cdf);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

int trust_tc_gen_er_device(trust_tc_ctx *ctx, int64_t n, int64_t npairs, uint64_t seed, int32_t *d_pairs) {
  if (n < 1 || n >= ((int64_t)1 << 31) || npairs < 0 || (npairs && !d_pairs)) return TRUST_TC_E_ARG;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  if (npairs) {
    er_kernel<<<gen_grid(npairs), 256>>>(n, npairs, gen_key(seed), d_pairs);
    TC_NOTE_LAUNCH();
  }
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaDeviceSynchronize());
  return TRUST_TC_OK;
}

int trust_tc_gen_ba_device(trust_tc_ctx *ctx, int64_t n, int d, uint64_t seed, int32_t *d_pairs) {
  if (n < 1 || n >= ((int64_t)1 << 31) || d < 1 || n * (int64_t)d >= ((int64_t)1 << 40) || !d_pairs)
    return TRUST_TC_E_ARG;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  const int64_t np = n * (int64_t)d;
  ba_kernel<<<gen_grid(np), 256>>>(np, d, gen_key(seed), d_pairs);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaDeviceSynchronize());
  return TRUST_TC_OK;
}

}  // extern "C"

// tc_split.cu — the direction split used by the learned schedule.
//
// The counted quantity sums, over arcs (v,u), |N+(v) ∩ N+(u)|.  The reference always hashes the
// source row N+(v) and streams the neighbour row N+(u) (Without-graph-partition/TC.cu:280-358), so
// an arc costs d(u) probes.  When rows are duplicate-free the intersection is symmetric, so an
// arc can instead be charged to its neighbour: hash N+(u) once and stream N+(v) for every source
// v that points at u, costing d(v) probes.  The split sends each arc with d(u) > d(v) to that
// second pass; the total probe count drops from sum d(u) to sum min(d(u), d(v)).  Only which row
// is hashed changes; the integer result is identical.
//
// Pass B needs, for each u, the sources v of its arcs sent to B: an in-list built here by a
// count / scan / scatter over the arcs (the order inside an in-list is irrelevant to the count).
#include <string.h>

#include <algorithm>

#include "tc_count.h"
#include "tc_internal.h"
#include "tc_model.h"

namespace tc {

// Rows strictly increasing (sorted, no duplicates)?  Clears nothing; sets TC_DEV_UNSORTED.
__global__ void rows_sorted_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                   TcControl *ctl) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int bad = 0;
  for (int64_t v = warp; v < n; v += nwarps) {
    const int64_t b = tc_ld_nc(beg + v), e = tc_ld_nc(beg + v + 1);
    for (int64_t i = b + lane; i + 1 < e; i += 32) bad |= tc_ld_nc(adj + i) >= tc_ld_nc(adj + i + 1);
  }
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  if (lane == 0 && bad) atomicOr(&ctl->status, TC_DEV_UNSORTED);
}

// Position (0..31) of the n-th (0-based) set bit of mask; mask must have more than n set bits.
__device__ __forceinline__ int split_nth_bit(unsigned mask, int n) {
  int pos = 0;
#pragma unroll
  for (int step = 16; step >= 1; step >>= 1) {
    const int cnt = __popc(mask & ((1u << step) - 1u));
    if (n >= cnt) {
      n -= cnt;
      mask >>= step;
      pos += step;
    }
  }
  return pos;
}

// Visit every arc (v,u) with d(v) >= 2 as f(v, d(v), u, d(u)).  A warp takes 32 consecutive
// vertices; rows of up to SPLIT_FLAT entries are flattened into one list over the 32 lanes
// (coalesced row reads, every lane's neighbour-degree loads independent), longer rows are walked
// by the whole warp.
constexpr int SPLIT_FLAT = 128;
template <class F>
__device__ __forceinline__ void for_each_arc(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                                             int64_t n, F f) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned upto = 0xffffffffu >> (31 - lane);
  for (int64_t v0 = warp * 32; v0 < n; v0 += nwarps * 32) {
    const int64_t v = v0 + lane;
    int b = 0, dv = 0;
    if (v < n) {
      const long long lo = tc_ld_nc(beg + v);
      b = (int)lo;
      dv = (int)(tc_ld_nc(beg + v + 1) - lo);
    }
    const int sd = (dv >= 2 && dv <= SPLIT_FLAT) ? dv : 0;
    // long rows
    unsigned big = __ballot_sync(TC_FULL_MASK, dv > SPLIT_FLAT);
    while (big) {
      const int j = __ffs(big) - 1;
      big &= big - 1;
      const int bj = __shfl_sync(TC_FULL_MASK, b, j);
      const int dj = __shfl_sync(TC_FULL_MASK, dv, j);
      for (int i = lane; i < dj; i += 32) {
        const int u = tc_ld_nc(adj + bj + i);
        f((int)(v0 + j), dj, u, (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u)));
      }
    }
    // short rows, flattened: ranked nonempty rows, owner of a slot from the start-bit mask
    int incl = sd;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(TC_FULL_MASK, incl, o);
      if (lane >= o) incl += y;
    }
    const int tot = __shfl_sync(TC_FULL_MASK, incl, 31);
    if (tot == 0) continue;
    const unsigned ne = __ballot_sync(TC_FULL_MASK, sd > 0);
    const int nc = __popc(ne);
    const int src = lane < nc ? split_nth_bit(ne, lane) : 0;
    const int src_excl = __shfl_sync(TC_FULL_MASK, incl - sd, src);
    const int cexcl = lane < nc ? src_excl : 0x7fffffff;
    const int cbase = __shfl_sync(TC_FULL_MASK, b - (incl - sd), src);
    const int cdeg = __shfl_sync(TC_FULL_MASK, sd, src);
    int before = 0;
    for (int k0 = 0; k0 < tot; k0 += 32) {
      const unsigned starts =
          __reduce_or_sync(TC_FULL_MASK, (cexcl >= k0 && cexcl < k0 + 32) ? (1u << (cexcl - k0)) : 0u);
      const int c = max(before + __popc(starts & upto) - 1, 0);
      before += __popc(starts);
      const int base = __shfl_sync(TC_FULL_MASK, cbase, c);
      const int deg = __shfl_sync(TC_FULL_MASK, cdeg, c);
      const int row = __shfl_sync(TC_FULL_MASK, src, c);
      const int k = k0 + lane;
      if (k < tot) {
        const int u = tc_ld_nc(adj + base + k);
        f((int)(v0 + row), deg, u, (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u)));
      }
    }
  }
}

// Scatter the sources of the second-pass arcs into their targets' in-lists.
__global__ void split_fill_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                  unsigned *__restrict__ cursor, const int64_t *__restrict__ off,
                                  int32_t *__restrict__ adj_b) {
  for_each_arc(beg, adj, n, [&](int v, int dv, int u, int du) {
    if (du > dv) adj_b[off[u] + atomicAdd(cursor + u, 1u)] = v;
  });
}

// ---- the learned schedule's scheduling pass ----------------------------------------------------
// MLP evaluated by a whole warp: lane j owns hidden unit j of both layers.  x: the 8 raw
// features, identical in every lane.  Returns the predicted log2 cycles in every lane.
// P is the packed model in shared memory with W1 and W2 stored transposed (input-major), so the
// 32 lanes read 32 consecutive floats (no bank conflicts).
__device__ __forceinline__ float warp_mlp(const float *__restrict__ P, const float *x_raw, int lane) {
  float x[TC_FEATURES];
#pragma unroll
  for (int i = 0; i < TC_FEATURES; ++i) x[i] = (x_raw[i] - P[TC_OFF_MEAN + i]) * P[TC_OFF_ISCALE + i];
  float a = P[TC_OFF_B1 + lane];
#pragma unroll
  for (int i = 0; i < TC_FEATURES; ++i) a += P[TC_OFF_W1 + i * TC_HIDDEN + lane] * x[i];
  const float h1 = a > 0.f ? a : 0.f;
  float b = P[TC_OFF_B2 + lane];
#pragma unroll 8
  for (int i = 0; i < TC_HIDDEN; ++i) b += P[TC_OFF_W2 + i * TC_HIDDEN + lane] * __shfl_sync(TC_FULL_MASK, h1, i);
  const float h2 = b > 0.f ? b : 0.f;
  float y = P[TC_OFF_W3 + lane] * h2;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) y += __shfl_xor_sync(TC_FULL_MASK, y, o);
  y += P[TC_OFF_B3];
  return y * P[TC_OFF_YSCALE] + P[TC_OFF_YMEAN];
}

// fp32 throughout: the FP64 rate of this part is a small fraction of its FP32 rate
__device__ __forceinline__ float flog2p1(float x) { return log2f(1.f + x); }

// The 8 features of a row (see include/trust_tc.h), from its warp-reduced statistics.
__device__ __forceinline__ void row_features(float *f, int dv, unsigned long long w, unsigned long long wmin,
                                             int maxdu, int nb, int cls) {
  f[0] = flog2p1((float)dv);
  f[1] = flog2p1((float)w);
  f[2] = flog2p1((float)wmin);
  f[3] = flog2p1((float)maxdu);
  f[4] = flog2p1((float)nb);
  f[5] = flog2p1((float)w / (float)max(dv, 1));
  f[6] = (float)cls;
  int t = 6;
  while ((1 << t) < 2 * dv) ++t;
  f[7] = (float)t;
}

__device__ __forceinline__ int tuned_class_of(int d, int warp_max, int cta_max) {
  if (d < 2) return TC_CLASS_SKIP;
  if (d <= 4) return TC_CLASS_G4;
  if (d <= 8) return TC_CLASS_G8;
  if (d <= 16) return TC_CLASS_G16;
  if (d <= 32) return TC_CLASS_G32;
  if (d <= warp_max) return TC_CLASS_WARP;
  return d <= cta_max ? TC_CLASS_CTA : TC_CLASS_HUGE;
}

// One traversal: the split plan's totals and in-list counts for every arc, and for every row
// longer than 32 its features, its predicted cycles (model) and its class decision: a warp-class
// row predicted to cost more than 2^promote_log2 cycles is promoted to a CTA.  sums[0] collects
// the predicted cycles the split would save (each row's prediction times its probe saving).
template <bool MODEL>
__global__ void sched_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                             unsigned *__restrict__ cnt, unsigned long long *__restrict__ wsum,
                             unsigned long long *plans, const float *__restrict__ model, int warp_max, int cta_max,
                             float promote_log2, unsigned char *__restrict__ dec, float *__restrict__ pred,
                             float *sums, float *__restrict__ feats, int cta_warps) {
  __shared__ float P[MODEL ? TC_MODEL_FLOATS : 1];
  if (MODEL) {  // staged with W1 and W2 transposed (see warp_mlp)
    for (int i = threadIdx.x; i < TC_MODEL_FLOATS; i += blockDim.x) {
      float v = model[i];
      if (i >= TC_OFF_W1 && i < TC_OFF_B1) {
        const int j = (i - TC_OFF_W1) / TC_FEATURES, k = (i - TC_OFF_W1) % TC_FEATURES;
        P[TC_OFF_W1 + k * TC_HIDDEN + j] = v;
      } else if (i >= TC_OFF_W2 && i < TC_OFF_B2) {
        const int j = (i - TC_OFF_W2) / TC_HIDDEN, k = (i - TC_OFF_W2) % TC_HIDDEN;
        P[TC_OFF_W2 + k * TC_HIDDEN + j] = v;
      } else {
        P[i] = v;
      }
    }
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned upto = 0xffffffffu >> (31 - lane);
  unsigned long long w_all = 0, w_min = 0;
  float saved = 0.f;
  for (int64_t v0 = warp * 32; v0 < n; v0 += nwarps * 32) {
    const int64_t v = v0 + lane;
    int b = 0, dv = 0;
    if (v < n) {
      const long long lo = tc_ld_nc(beg + v);
      b = (int)lo;
      dv = (int)(tc_ld_nc(beg + v + 1) - lo);
    }
    // rows longer than 32: a warp each, with features and the model
    unsigned big = __ballot_sync(TC_FULL_MASK, dv > 32);
    while (big) {
      const int j = __ffs(big) - 1;
      big &= big - 1;
      const int bj = __shfl_sync(TC_FULL_MASK, b, j);
      const int dj = __shfl_sync(TC_FULL_MASK, dv, j);
      unsigned long long rw = 0, rmin = 0;
      int rmax = 0, rnb = 0;
      for (int i = lane; i < dj; i += 32) {
        const int u = tc_ld_nc(adj + bj + i);
        const int du = (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u));
        rw += (unsigned)du;
        rmin += (unsigned)min(du, dj);
        rmax = max(rmax, du);
        if (du > dj) {
          ++rnb;
          atomicAdd(cnt + u, 1u);
          atomicAdd(wsum + u, (unsigned long long)dj);
        }
      }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        rw += __shfl_xor_sync(TC_FULL_MASK, rw, o);
        rmin += __shfl_xor_sync(TC_FULL_MASK, rmin, o);
        rmax = max(rmax, __shfl_xor_sync(TC_FULL_MASK, rmax, o));
        rnb += __shfl_xor_sync(TC_FULL_MASK, rnb, o);
      }
      if (lane == 0) {
        w_all += rw;
        w_min += rmin;
      }
      const int cls = tuned_class_of(dj, warp_max, cta_max);
      float f[TC_FEATURES];
      row_features(f, dj, rw, rmin, rmax, rnb, cls);
      if (feats && lane < TC_FEATURES) feats[(v0 + j) * TC_FEATURES + lane] = f[lane];
      if (MODEL) {
        const float y = warp_mlp(P, f, lane);
        if (lane == 0) {
          int d = cls;
          if (d == TC_CLASS_WARP && y > promote_log2) d = TC_CLASS_CTA;
          dec[v0 + j] = (unsigned char)d;
          pred[v0 + j] = y;
          // warp-cycles: a CTA row's cycles are spent by all its warps
          const float warps = d >= TC_CLASS_CTA ? (float)cta_warps : 1.f;
          if (rw > 0) saved += warps * exp2f(fminf(y, 60.f)) * (float)((double)(rw - rmin) / (double)rw);
        }
      }
    }
    // rows of 2..32 entries: flattened over the warp (split totals and counts only)
    const int sd = (dv >= 2 && dv <= 32) ? dv : 0;
    int incl = sd;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(TC_FULL_MASK, incl, o);
      if (lane >= o) incl += y;
    }
    const int tot = __shfl_sync(TC_FULL_MASK, incl, 31);
    if (tot == 0) continue;
    const unsigned ne = __ballot_sync(TC_FULL_MASK, sd > 0);
    const int nc = __popc(ne);
    const int src = lane < nc ? split_nth_bit(ne, lane) : 0;
    const int src_excl = __shfl_sync(TC_FULL_MASK, incl - sd, src);
    const int cexcl = lane < nc ? src_excl : 0x7fffffff;
    const int cbase = __shfl_sync(TC_FULL_MASK, b - (incl - sd), src);
    const int cdeg = __shfl_sync(TC_FULL_MASK, sd, src);
    int before = 0;
    for (int k0 = 0; k0 < tot; k0 += 32) {
      const unsigned starts =
          __reduce_or_sync(TC_FULL_MASK, (cexcl >= k0 && cexcl < k0 + 32) ? (1u << (cexcl - k0)) : 0u);
      const int c = max(before + __popc(starts & upto) - 1, 0);
      before += __popc(starts);
      const int base = __shfl_sync(TC_FULL_MASK, cbase, c);
      const int deg = __shfl_sync(TC_FULL_MASK, cdeg, c);
      const int k = k0 + lane;
      if (k < tot) {
        const int u = tc_ld_nc(adj + base + k);
        const int du = (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u));
        w_all += (unsigned)du;
        w_min += (unsigned)min(du, deg);
        if (du > deg) {
          atomicAdd(cnt + u, 1u);
          atomicAdd(wsum + u, (unsigned long long)deg);
        }
      }
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    w_all += __shfl_down_sync(TC_FULL_MASK, w_all, o);
    w_min += __shfl_down_sync(TC_FULL_MASK, w_min, o);
    saved += __shfl_down_sync(TC_FULL_MASK, saved, o);
  }
  if (lane == 0) {
    atomicAdd(plans + 0, w_all);
    atomicAdd(plans + 1, w_min);
    if (MODEL && saved > 0.f) atomicAdd(sums, saved);
  }
}

__global__ void u32_to_i64_kernel(const unsigned *__restrict__ in, int64_t *__restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// Work rows of target u: each rebuilds u's table (about 3 d(u) operations), so u's incoming
// probe work W_B(u) = sum of d(v) over its sources is cut into pieces of at least
// max(TC_SPLIT_WORK_PER_ENTRY * d(u), TC_SPLIT_MIN_WORK) probes, with equal source counts.
__device__ __forceinline__ int64_t chunks_of(unsigned cnt, unsigned long long w, int du) {
  if (cnt == 0) return 0;
  const unsigned long long target =
      max((unsigned long long)TC_SPLIT_WORK_PER_ENTRY * (unsigned long long)du, (unsigned long long)TC_SPLIT_MIN_WORK);
  const unsigned long long k = (w + target - 1) / target;
  return (int64_t)min(max(k, 1ull), (unsigned long long)cnt);
}

// chunks per target; the last entry (index n) is 0
__global__ void chunk_count_kernel(const int64_t *__restrict__ beg, const unsigned *__restrict__ cnt,
                                   const unsigned long long *__restrict__ wsum, int64_t *__restrict__ nch,
                                   int64_t n) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u <= n; u += (int64_t)gridDim.x * blockDim.x)
    nch[u] = u < n ? chunks_of(cnt[u], wsum[u], (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u))) : 0;
}

// work rows: chunk j of target u covers in-list entries [off[u] + j S, off[u] + (j+1) S) with
// S = ceil(cnt / chunks) (the last one ends at the next row's start); rowmap[k] = u
__global__ void chunk_fill_kernel(const int64_t *__restrict__ cbase, const int64_t *__restrict__ off, int64_t n,
                                  int64_t total, int64_t nchunks, int64_t *__restrict__ cbeg,
                                  int *__restrict__ rowmap) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k0 = cbase[u], k1 = cbase[u + 1];
    if (k0 == k1) continue;
    const int64_t cnt = off[u + 1] - off[u];
    const int64_t S = (cnt + (k1 - k0) - 1) / (k1 - k0);
    for (int64_t k = k0; k < k1; ++k) {
      cbeg[k] = min(off[u] + (k - k0) * S, off[u + 1]);
      rowmap[k] = (int)u;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cbeg[nchunks] = total;
}

int launch_rows_sorted(const int64_t *beg, const int32_t *adj, int64_t n, TcControl *ctl, int num_sms, cudaStream_t st) {
  int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, (int64_t)num_sms * 8));
  rows_sorted_kernel<<<blocks, 256, 0, st>>>(beg, adj, n, ctl);
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

static int arc_blocks(int64_t n, int num_sms) {  // one warp per 32 vertices
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 16));
}

// The scheduling pass (one traversal of the arcs): probe totals of both plans, the split's
// in-degree counts and work sums, and - with a model - every long row's predicted cycles and
// class decision plus the predicted saving of the split (SchedPlan).
int split_plan(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, cudaStream_t st,
               const float *d_model, int warp_max, int cta_max, float promote_log2, SchedPlan *plan,
               float *d_features, int cta_warps) {
  int rc = ensure((void **)&c->d_split_cnt, &c->split_cnt_cap, sizeof(unsigned) * (size_t)std::max<int64_t>(n + 1, 1));
  if (rc) return rc;
  rc = ensure((void **)&c->d_split_plans, &c->split_plans_cap, 4 * sizeof(unsigned long long));
  if (rc) return rc;
  rc = ensure((void **)&c->d_split_wsum, &c->split_wsum_cap, sizeof(unsigned long long) * (size_t)(n + 1));
  if (rc) return rc;
  if (d_model) {
    if ((rc = ensure((void **)&c->d_dec, &c->dec_cap, (size_t)std::max<int64_t>(n, 1)))) return rc;
    if ((rc = ensure((void **)&c->d_pred, &c->pred_cap, sizeof(float) * (size_t)std::max<int64_t>(n, 1)))) return rc;
  }
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_cnt, 0, sizeof(unsigned) * (size_t)(n + 1), st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_wsum, 0, sizeof(unsigned long long) * (size_t)(n + 1), st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_plans, 0, 4 * sizeof(unsigned long long), st));
  float *sums = reinterpret_cast<float *>(c->d_split_plans + 2);
  const int blocks = arc_blocks(n, c->num_sms);
  if (d_model)
    sched_kernel<true><<<blocks, 256, 0, st>>>(beg, adj, n, c->d_split_cnt, c->d_split_wsum, c->d_split_plans, d_model,
                                               warp_max, cta_max, promote_log2, c->d_dec, c->d_pred, sums, d_features,
                                               cta_warps);
  else
    sched_kernel<false><<<blocks, 256, 0, st>>>(beg, adj, n, c->d_split_cnt, c->d_split_wsum, c->d_split_plans,
                                                nullptr, warp_max, cta_max, promote_log2, nullptr, nullptr, nullptr,
                                                d_features, cta_warps);
  TC_CUDA_TRY(cudaGetLastError());
  unsigned long long hp[4];
  TC_CUDA_TRY(cudaMemcpyAsync(hp, c->d_split_plans, sizeof hp, cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  plan->w_all = hp[0];
  plan->w_min = hp[1];
  float saved = 0.f;
  memcpy(&saved, &hp[2], sizeof saved);
  plan->saved_cycles = saved;
  return TRUST_TC_OK;
}

// Build the second pass's work rows (after split_plan): the in-list of every target, cut into
// chunks (chunk_len) so one heavily targeted row spreads over many CTAs.
// Outputs live in the context.
int split_build(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, cudaStream_t st,
                SplitRows *out) {
  const int64_t max_chunks = std::max<int64_t>(n, m) + 1;  // at most one chunk per source
  int rc;
  if ((rc = ensure((void **)&c->d_split_beg, &c->split_beg_cap, sizeof(int64_t) * (size_t)(n + 1)))) return rc;
  if ((rc = ensure((void **)&c->d_split_cbase, &c->split_cbase_cap, sizeof(int64_t) * (size_t)(n + 1)))) return rc;
  if ((rc = ensure((void **)&c->d_split_cbeg, &c->split_cbeg_cap, sizeof(int64_t) * (size_t)(max_chunks + 1)))) return rc;
  if ((rc = ensure((void **)&c->d_split_rowmap, &c->split_rowmap_cap, sizeof(int) * (size_t)max_chunks))) return rc;
  if ((rc = ensure((void **)&c->d_split_adj, &c->split_adj_cap, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1))))
    return rc;
  const int vb = arc_blocks(n + 1, c->num_sms);
  // in-list offsets: exclusive scan of the in-degrees (entry n is 0)
  u32_to_i64_kernel<<<vb, 256, 0, st>>>(c->d_split_cnt, c->d_split_beg, n + 1);
  TC_CUDA_TRY(cudaGetLastError());
  int64_t total = 0;
  if ((rc = scan_exclusive_i64(c->d_split_beg, c->d_split_beg, n + 1, st, &total))) return rc;
  if (total > m) return TRUST_TC_E_DEVICE;
  // chunk bases
  chunk_count_kernel<<<vb, 256, 0, st>>>(beg, c->d_split_cnt, c->d_split_wsum, c->d_split_cbase, n);
  TC_CUDA_TRY(cudaGetLastError());
  int64_t nchunks = 0;
  if ((rc = scan_exclusive_i64(c->d_split_cbase, c->d_split_cbase, n + 1, st, &nchunks))) return rc;
  if (nchunks > max_chunks) return TRUST_TC_E_DEVICE;
  // scatter the sources
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_cnt, 0, sizeof(unsigned) * (size_t)(n + 1), st));
  split_fill_kernel<<<arc_blocks(n, c->num_sms), 256, 0, st>>>(beg, adj, n, c->d_split_cnt, c->d_split_beg,
                                                               c->d_split_adj);
  TC_CUDA_TRY(cudaGetLastError());
  chunk_fill_kernel<<<vb, 256, 0, st>>>(c->d_split_cbase, c->d_split_beg, n, total, nchunks, c->d_split_cbeg,
                                        c->d_split_rowmap);
  TC_CUDA_TRY(cudaGetLastError());
  out->beg = c->d_split_cbeg;
  out->adj = c->d_split_adj;
  out->rowmap = c->d_split_rowmap;
  out->rows = nchunks;
  out->m = total;
  return TRUST_TC_OK;
}

// ---- heaviest-first queue order ------------------------------------------------------------------
__global__ void lpt_keys_kernel(const int *__restrict__ list, int count, const float *__restrict__ pred,
                                unsigned long long *__restrict__ keys) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const int v = list[i];
    const float y = fminf(fmaxf(pred[v], 0.f), 63.9f);
    const unsigned q = 65535u - (unsigned)(y * 1024.f);  // larger prediction sorts first
    keys[i] = ((unsigned long long)q << 32) | (unsigned)v;
  }
}

__global__ void lpt_store_kernel(const unsigned long long *__restrict__ keys, int count, int *__restrict__ list) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    list[i] = (int)(keys[i] & 0xffffffffu);
}

int lpt_sort(trust_tc_ctx *c, int *lists, const int *off, const int *counts, const float *pred, cudaStream_t st) {
  const int classes[3] = {TC_CLASS_HUGE, TC_CLASS_CTA, TC_CLASS_WARP};
  int64_t most = 0;
  for (int k : classes) most = std::max<int64_t>(most, counts[k]);
  if (most < 2) return TRUST_TC_OK;
  int rc = ensure((void **)&c->d_sort, &c->sort_cap, sizeof(unsigned long long) * 2 * (size_t)most);
  if (rc) return rc;
  const int shifts[2] = {32, 40};  // the 16-bit cost key only; the sort is stable
  for (int k : classes) {
    const int cnt = counts[k];
    if (cnt < 2) continue;
    const int blocks = std::max(1, std::min((cnt + 255) / 256, c->num_sms * 8));
    lpt_keys_kernel<<<blocks, 256, 0, st>>>(lists + off[k], cnt, pred, c->d_sort);
    TC_CUDA_TRY(cudaGetLastError());
    rc = radix_sort_u64(c->d_sort, c->d_sort + most, cnt, shifts, 2, st);
    if (rc) return rc;
    lpt_store_kernel<<<blocks, 256, 0, st>>>(c->d_sort, cnt, lists + off[k]);
    TC_CUDA_TRY(cudaGetLastError());
  }
  return TRUST_TC_OK;
}

// ---- features of every vertex (training data) ----------------------------------------------------
__global__ void vertex_features_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                       int warp_max, int cta_max, float *__restrict__ feats) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    const int64_t b = tc_ld_nc(beg + v);
    const int dv = (int)(tc_ld_nc(beg + v + 1) - b);
    float f[TC_FEATURES];
    if (dv < 2) {
      if (lane < TC_FEATURES) feats[v * TC_FEATURES + lane] = 0.f;
      continue;
    }
    unsigned long long rw = 0, rmin = 0;
    int rmax = 0, rnb = 0;
    for (int i = lane; i < dv; i += 32) {
      const int u = tc_ld_nc(adj + b + i);
      const int du = (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u));
      rw += (unsigned)du;
      rmin += (unsigned)min(du, dv);
      rmax = max(rmax, du);
      rnb += du > dv;
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      rw += __shfl_xor_sync(TC_FULL_MASK, rw, o);
      rmin += __shfl_xor_sync(TC_FULL_MASK, rmin, o);
      rmax = max(rmax, __shfl_xor_sync(TC_FULL_MASK, rmax, o));
      rnb += __shfl_xor_sync(TC_FULL_MASK, rnb, o);
    }
    row_features(f, dv, rw, rmin, rmax, rnb, tuned_class_of(dv, warp_max, cta_max));
    if (lane < TC_FEATURES) feats[v * TC_FEATURES + lane] = f[lane];
  }
}

int vertex_features(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int warp_max, int cta_max,
                    float *d_features, cudaStream_t st) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, (int64_t)c->num_sms * 16));
  vertex_features_kernel<<<blocks, 256, 0, st>>>(beg, adj, n, warp_max, cta_max, d_features);
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

}  // namespace tc

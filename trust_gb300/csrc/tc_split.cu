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

// ---- traversal of the arcs ---------------------------------------------------------------------
// Every arc (v,u) with d(v) >= 2 is visited once, in two phases.  Phase 1: a warp takes 32
// consecutive vertices and flattens their rows of 2..TC_SCHED_FLAT entries into one list over
// the lanes (coalesced row reads, independent neighbour-degree loads); longer rows are appended
// to a list.  Phase 2: one warp per listed row, rows dealt round-robin over the warps, four
// 32-entry steps of loads in flight.  No warp walks a whole tile of long rows (after renumbering
// by out-degree the first tiles hold the longest rows of the graph).
constexpr int TC_SCHED_FLAT = 32;

// Phase 1.  f(valid, v, d(v), u, d(u), pos, last) is called by all 32 lanes together (warp
// collectives allowed); lanes with valid = false carry no arc.  pos = the arc's index in adj,
// last = it ends its row.  Rows longer than TC_SCHED_FLAT are appended to longs[] (length in
// *nlong) when longs is given.  Rows outside [row_lo, row_hi) are passed over.
template <class F>
__device__ __forceinline__ void short_arcs(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                                           int64_t n, int64_t row_lo, int64_t row_hi, int *__restrict__ longs,
                                           unsigned long long *nlong, F f) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned upto = 0xffffffffu >> (31 - lane);
  for (int64_t v0 = warp * 32; v0 < n; v0 += nwarps * 32) {
    const int64_t v = v0 + lane;
    int b = 0, dv = 0;
    if (v < n && v >= row_lo && v < row_hi) {
      const long long lo = tc_ld_nc(beg + v);
      b = (int)lo;
      dv = (int)(tc_ld_nc(beg + v + 1) - lo);
    }
    if (longs) {
      const unsigned big = __ballot_sync(TC_FULL_MASK, dv > TC_SCHED_FLAT);
      if (big) {
        unsigned long long at = 0;
        if (lane == 0) at = atomicAdd(nlong, (unsigned long long)__popc(big));
        at = __shfl_sync(TC_FULL_MASK, at, 0);
        if (dv > TC_SCHED_FLAT) longs[at + __popc(big & (upto >> 1))] = (int)v;
      }
    }
    // ranked nonempty rows; the owner of a slot comes from the start-bit mask
    const int sd = (dv >= 2 && dv <= TC_SCHED_FLAT) ? dv : 0;
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
      const int ex = __shfl_sync(TC_FULL_MASK, cexcl, c);
      const int row = __shfl_sync(TC_FULL_MASK, src, c);
      const int k = k0 + lane;
      const bool valid = k < tot;
      const int pos = base + k;
      int u = 0, du = 0;
      if (valid) {
        u = tc_ld_nc(adj + pos);
        du = (int)(tc_ld_nc(beg + u + 1) - tc_ld_nc(beg + u));
      }
      f(valid, (int)(v0 + row), deg, u, du, pos, k + 1 == ex + deg);
    }
  }
}

// Phase 2 for one row (entries adj[b, b+dv)) by a whole warp: f(valid, u, d(u), pos, last), called
// by all lanes together as in phase 1.
template <class F>
__device__ __forceinline__ void long_row_arcs(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                                              int b, int dv, int lane, F f) {
  for (int i0 = 0; i0 < dv; i0 += 128) {
    int u[4], du[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = i0 + 32 * k + lane;
      u[k] = i < dv ? tc_ld_nc(adj + b + i) : -1;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) du[k] = u[k] >= 0 ? (int)(tc_ld_nc(beg + u[k] + 1) - tc_ld_nc(beg + u[k])) : 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = i0 + 32 * k + lane;
      f(i < dv, u[k], du[k], b + i, i == dv - 1);
    }
  }
}

// Pair slots are reserved TC_PAIR_BLOCK at a time per warp (one atomic on the shared slot counter
// per block, not one per 32-arc step: every warp of the pass hits that counter).  A warp abandons
// the rest of a block when a step's pairs do not fit, and at its end; abandoned slots are holes
// (x = -1) that the fill skips.  Slots used <= moved arcs * TC_PAIR_BLOCK / (TC_PAIR_BLOCK - 31)
// + TC_PAIR_BLOCK per warp (pair_slots() below).
constexpr unsigned TC_PAIR_BLOCK = 256;
struct PairBuf {
  unsigned long long next = 0;  // warp-uniform: next free slot of the current block
  unsigned avail = 0;           // slots left in it
  unsigned long long cap;       // slots in the pair arrays; 0 once a reservation would pass them
  unsigned long long *overflow; // set (never expected: the arrays hold pair_slots()) and no more pairs
};

__device__ __forceinline__ void pair_holes(PairBuf &pb, int2 *__restrict__ pairs) {
  for (unsigned i = threadIdx.x & 31; i < pb.avail; i += 32) pairs[pb.next + i].x = -1;
  pb.next += pb.avail;
  pb.avail = 0;
}

// An arc (v,u) the split would move (mv): count it in u's in-list (cnt) and work sum (wsum) and
// append it as a (target, source) pair; the fill gives each pair its slot in u's in-list.  The
// counts are reductions whose result nobody waits for, so a step of the pass never stalls on an
// atomic's round trip.  Called by all 32 lanes together; lanes that move an arc to the same target
// share one atomic (hub targets receive many).
__device__ __forceinline__ void move_arc(bool mv, int u, int v, int dv, unsigned *__restrict__ cnt,
                                         unsigned long long *__restrict__ wsum, int2 *__restrict__ pairs,
                                         unsigned long long *npairs, PairBuf &pb) {
  const unsigned m = __ballot_sync(TC_FULL_MASK, mv);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const unsigned lt = tc_lanemask_lt();
  const unsigned peers = __match_any_sync(TC_FULL_MASK, mv ? u : -1);
  if (mv) {
    const unsigned sum = __reduce_add_sync(peers, (unsigned)dv);
    if ((peers & lt) == 0) {  // the group's leader
      atomicAdd(cnt + u, (unsigned)__popc(peers));
      atomicAdd(wsum + u, (unsigned long long)sum);
    }
  }
  const unsigned k = __popc(m);
  if (pb.cap == 0) return;
  if (k > pb.avail) {  // warp-uniform
    pair_holes(pb, pairs);
    unsigned long long at = 0;
    if (lane == 0) at = atomicAdd(npairs, (unsigned long long)TC_PAIR_BLOCK);
    at = __shfl_sync(TC_FULL_MASK, at, 0);
    if (at + TC_PAIR_BLOCK > pb.cap) {
      if (lane == 0) atomicOr(pb.overflow, 1ull);
      pb.cap = 0;
      return;
    }
    pb.next = at;
    pb.avail = TC_PAIR_BLOCK;
  }
  if (mv) pairs[pb.next + __popc(m & lt)] = make_int2(u, v);
  pb.next += k;
  pb.avail -= k;
}

// Fill the in-lists: every pair's source goes to the next free slot of its target's in-list
// (cursor: one counter per target, zeroed before), holes skipped; four pairs per thread in
// flight, so the cursor atomics' round trips overlap.
__global__ void split_fill_kernel(const int2 *__restrict__ pairs, const unsigned long long *__restrict__ npairs,
                                  const int64_t *__restrict__ off, unsigned *__restrict__ cursor,
                                  int32_t *__restrict__ adj_b) {
  const int64_t np = (int64_t)*npairs;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < np; i += 4 * stride) {
    int2 p[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) p[r] = i + r * stride < np ? pairs[i + r * stride] : make_int2(-1, 0);
    unsigned slot[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) slot[r] = p[r].x >= 0 ? atomicAdd(cursor + p[r].x, 1u) : 0u;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (p[r].x >= 0) adj_b[off[p[r].x] + slot[r]] = p[r].y;
  }
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

// Words of the scheduling pass's totals (plans[]).
enum { PLAN_W_ALL = 0, PLAN_W_MIN = 1, PLAN_SAVED = 2, PLAN_NLONG = 3, PLAN_NPAIRS = 4, PLAN_OVERFLOW = 5 };

// The scheduling pass, phase 1 (rows of up to TC_SCHED_FLAT entries): the split plan's probe
// totals, the in-list count and work sum of every arc's target, the arcs the split would move
// (as pairs), and the sortedness check; rows longer than TC_SCHED_FLAT are listed.
__global__ void sched_short_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                   int64_t row_lo, int64_t row_hi, unsigned *__restrict__ cnt,
                                   unsigned long long *__restrict__ wsum, unsigned long long *plans,
                                   int *__restrict__ longs, int2 *__restrict__ pairs, unsigned long long pair_cap,
                                   TcControl *ctl) {
  const int lane = threadIdx.x & 31;
  unsigned long long w_all = 0, w_min = 0;
  int bad = 0;
  PairBuf pb;
  pb.cap = pair_cap;
  pb.overflow = plans + PLAN_OVERFLOW;
  short_arcs(beg, adj, n, row_lo, row_hi, longs, plans + PLAN_NLONG,
             [&](bool valid, int v, int dv, int u, int du, int pos, bool last) {
               if (valid) {
                 w_all += (unsigned)du;
                 w_min += (unsigned)min(du, dv);
                 if (!last) bad |= u >= tc_ld_nc(adj + pos + 1);
               }
               move_arc(valid && du > dv, u, v, dv, cnt, wsum, pairs, plans + PLAN_NPAIRS, pb);
             });
  pair_holes(pb, pairs);
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    w_all += __shfl_down_sync(TC_FULL_MASK, w_all, o);
    w_min += __shfl_down_sync(TC_FULL_MASK, w_min, o);
  }
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  if (lane == 0) {
    if (w_all) atomicAdd(plans + PLAN_W_ALL, w_all);
    if (w_min) atomicAdd(plans + PLAN_W_MIN, w_min);
    if (bad) atomicOr(&ctl->status, TC_DEV_UNSORTED);
  }
}

// Phase 2 (the listed rows, a warp each): the same totals, counts and check, plus every row's
// features and, with a model, its predicted cycles and class decision: a warp-class row
// predicted to cost more than 2^promote_log2 cycles is promoted to a CTA.  sums[0] collects the
// predicted cycles the split would save (each row's prediction times its probe saving).
template <bool MODEL>
__global__ void sched_long_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                                  unsigned *__restrict__ cnt, unsigned long long *__restrict__ wsum,
                                  unsigned long long *plans, const int *__restrict__ longs,
                                  const float *__restrict__ model, int warp_max, int cta_max, float promote_log2,
                                  unsigned char *__restrict__ dec, float *__restrict__ pred, float *sums,
                                  int cta_warps, int2 *__restrict__ pairs, unsigned long long pair_cap,
                                  TcControl *ctl) {
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
  const int64_t nl = (int64_t)plans[PLAN_NLONG];
  unsigned long long w_all = 0, w_min = 0;
  float saved = 0.f;
  int bad = 0;
  PairBuf pb;
  pb.cap = pair_cap;
  pb.overflow = plans + PLAN_OVERFLOW;
  for (int64_t idx = warp; idx < nl; idx += nwarps) {
    const int v = longs[idx];
    const long long lo = tc_ld_nc(beg + v);
    const int dv = (int)(tc_ld_nc(beg + v + 1) - lo);
    unsigned long long rw = 0, rmin = 0;
    int rmax = 0, rnb = 0;
    long_row_arcs(beg, adj, (int)lo, dv, lane, [&](bool valid, int u, int du, int pos, bool last) {
      const bool mv = valid && du > dv;
      if (valid) {
        rw += (unsigned)du;
        rmin += (unsigned)min(du, dv);
        rmax = max(rmax, du);
        rnb += mv;
        if (!last) bad |= u >= tc_ld_nc(adj + pos + 1);
      }
      move_arc(mv, u, v, dv, cnt, wsum, pairs, plans + PLAN_NPAIRS, pb);
    });
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
    if (MODEL) {
      const int cls = tuned_class_of(dv, warp_max, cta_max);
      float f[TC_FEATURES];
      row_features(f, dv, rw, rmin, rmax, rnb, cls);
      const float y = warp_mlp(P, f, lane);
      if (lane == 0) {
        int d = cls;
        if (d == TC_CLASS_WARP && y > promote_log2) d = TC_CLASS_CTA;
        dec[v] = (unsigned char)d;
        pred[v] = y;
        // warp-cycles: a CTA row's cycles are spent by all its warps
        const float warps = d >= TC_CLASS_CTA ? (float)cta_warps : 1.f;
        if (rw > 0) saved += warps * exp2f(fminf(y, 60.f)) * (float)((double)(rw - rmin) / (double)rw);
      }
    }
  }
  pair_holes(pb, pairs);
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  if (lane == 0) {
    if (w_all) atomicAdd(plans + PLAN_W_ALL, w_all);
    if (w_min) atomicAdd(plans + PLAN_W_MIN, w_min);
    if (MODEL && saved > 0.f) atomicAdd(sums, saved);
    if (bad) atomicOr(&ctl->status, TC_DEV_UNSORTED);
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

static int arc_blocks(int64_t n, int num_sms) {  // one warp per 32 vertices
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 16));
}

// Pair slots for `arcs` arcs traversed by `warps` warps: a warp gives up a block only when fewer
// than 32 of its slots are left, so every block but a warp's last holds >= TC_PAIR_BLOCK - 31
// pairs: slots <= moved * 256 / 225 + 256 per warp <= arcs + arcs / 7 + 256 (warps + 1).
static size_t pair_slots(int64_t arcs, int64_t warps) {
  return (size_t)(arcs + arcs / 7) + (size_t)TC_PAIR_BLOCK * (size_t)(warps + 1);
}

// The scheduling pass (one traversal of the arcs, two phases): probe totals of both plans, the
// split's in-degree counts and work sums, the sortedness check (TC_DEV_UNSORTED in ctl), the list
// of rows longer than TC_SCHED_FLAT (kept for split_build), and - with a model - every long row's
// predicted cycles and class decision plus the predicted saving of the split.  Enqueued only:
// the totals reach the host with the stream's next synchronisation (split_plan_read).
int split_plan(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, cudaStream_t st,
               const float *d_model, int warp_max, int cta_max, float promote_log2, int cta_warps, TcControl *ctl,
               int64_t row_lo, int64_t row_hi) {
  const size_t nn = (size_t)std::max<int64_t>(n + 1, 1);
  int rc = ensure((void **)&c->d_split_cnt, &c->split_cnt_cap, sizeof(unsigned) * nn);
  if (rc) return rc;
  if ((rc = ensure((void **)&c->d_split_plans, &c->split_plans_cap, TC_PLAN_WORDS * sizeof(unsigned long long))))
    return rc;
  if ((rc = ensure((void **)&c->d_split_wsum, &c->split_wsum_cap, sizeof(unsigned long long) * nn))) return rc;
  if ((rc = ensure((void **)&c->d_sched_long, &c->sched_long_cap, sizeof(int) * nn))) return rc;
  const int sb = arc_blocks(n, c->num_sms), lb = c->num_sms * 8;  // 256-thread blocks of the two phases
  const size_t slots = pair_slots(m, (int64_t)(sb + lb) * 8);
  if ((rc = ensure((void **)&c->d_split_pairs, &c->split_pairs_cap, sizeof(int2) * slots))) return rc;
  if (d_model) {
    if ((rc = ensure((void **)&c->d_dec, &c->dec_cap, nn))) return rc;
    if ((rc = ensure((void **)&c->d_pred, &c->pred_cap, sizeof(float) * nn))) return rc;
  }
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_cnt, 0, sizeof(unsigned) * (size_t)(n + 1), st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_wsum, 0, sizeof(unsigned long long) * (size_t)(n + 1), st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_plans, 0, TC_PLAN_WORDS * sizeof(unsigned long long), st));
  float *sums = reinterpret_cast<float *>(c->d_split_plans + PLAN_SAVED);
  if (row_hi <= 0) row_hi = n;
  sched_short_kernel<<<sb, 256, 0, st>>>(beg, adj, n, row_lo, row_hi, c->d_split_cnt, c->d_split_wsum,
                                         c->d_split_plans, c->d_sched_long, c->d_split_pairs, slots, ctl);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  if (d_model)
    sched_long_kernel<true><<<lb, 256, 0, st>>>(beg, adj, c->d_split_cnt, c->d_split_wsum, c->d_split_plans,
                                                c->d_sched_long, d_model, warp_max, cta_max, promote_log2, c->d_dec,
                                                c->d_pred, sums, cta_warps, c->d_split_pairs, slots, ctl);
  else
    sched_long_kernel<false><<<lb, 256, 0, st>>>(beg, adj, c->d_split_cnt, c->d_split_wsum, c->d_split_plans,
                                                 c->d_sched_long, nullptr, warp_max, cta_max, promote_log2, nullptr,
                                                 nullptr, nullptr, cta_warps, c->d_split_pairs, slots, ctl);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaMemcpyAsync(c->h_plans, c->d_split_plans, TC_PLAN_WORDS * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, st));
  return TRUST_TC_OK;
}

void split_plan_read(const trust_tc_ctx *c, SchedPlan *plan) {
  plan->w_all = c->h_plans[PLAN_W_ALL];
  plan->w_min = c->h_plans[PLAN_W_MIN];
  float saved = 0.f;
  memcpy(&saved, &c->h_plans[PLAN_SAVED], sizeof saved);
  plan->saved_cycles = saved;
  plan->long_rows = (int64_t)c->h_plans[PLAN_NLONG];
  plan->moved_arcs = (int64_t)c->h_plans[PLAN_NPAIRS];  // pair slots used, holes included
  plan->overflow = c->h_plans[PLAN_OVERFLOW] != 0;
}

// ---- tile jobs: three CSRs ---------------------------------------------------------------------
// A tile job (i,j,k) hashes table rows A[v] (tile (i,j)), walks the arcs (v,u) of B[v] (tile
// (i,k)) and streams probe rows C[u] (tile (k,j)); an arc costs |C[u]| probes.  Counted from u's
// side (hash C[u], stream A[v]) it costs |A[v]|, and |A[v] ∩ C[u]| is the same number when both
// rows are duplicate-free.  The plan moves every arc with |C[u]| > |A[v]| of a row with A[v]
// nonempty (rows with A[v] empty contribute nothing from either side).  Tile rows are short (a
// quarter of a 2x2 split's row on average), so a warp takes 32 rows per step, as the whole-graph
// pass does.
__global__ void tile_sched_kernel(const int64_t *__restrict__ begA, const int64_t *__restrict__ begB,
                                  const int32_t *__restrict__ adjB, const int64_t *__restrict__ begC, int64_t rows,
                                  unsigned *__restrict__ cnt, unsigned long long *__restrict__ wsum,
                                  unsigned long long *plans, int2 *__restrict__ pairs, unsigned long long pair_cap) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned upto = 0xffffffffu >> (31 - lane);
  unsigned long long w_all = 0, w_min = 0;
  PairBuf pb;
  pb.cap = pair_cap;
  pb.overflow = plans + PLAN_OVERFLOW;
  auto arc = [&](bool valid, int v, int dA, int64_t pos) {  // all 32 lanes together
    int u = 0, du = 0;
    if (valid) {
      u = tc_ld_nc(adjB + pos);
      du = (int)(tc_ld_nc(begC + u + 1) - tc_ld_nc(begC + u));
      w_all += (unsigned)du;
      w_min += (unsigned)min(du, dA);
    }
    move_arc(valid && du > dA, u, v, dA, cnt, wsum, pairs, plans + PLAN_NPAIRS, pb);
  };
  // 32 consecutive rows per warp step: rows of up to 32 arcs flattened over the lanes (owner from
  // a start-bit mask, as in the whole-graph pass), longer rows walked by the warp one at a time
  for (int64_t v0 = warp * 32; v0 < rows; v0 += nwarps * 32) {
    const int64_t v = v0 + lane;
    long long b = 0;
    int dA = 0, dB = 0;
    if (v < rows) {
      dA = (int)(tc_ld_nc(begA + v + 1) - tc_ld_nc(begA + v));
      b = tc_ld_nc(begB + v);
      dB = dA >= 1 ? (int)(tc_ld_nc(begB + v + 1) - b) : 0;  // rows without a table contribute nothing
    }
    unsigned longs = __ballot_sync(TC_FULL_MASK, dB > 32);
    while (longs) {
      const int j = __ffs(longs) - 1;
      longs &= longs - 1;
      const long long bj = __shfl_sync(TC_FULL_MASK, b, j);
      const int dj = __shfl_sync(TC_FULL_MASK, dB, j);
      const int aj = __shfl_sync(TC_FULL_MASK, dA, j);
      for (int i0 = 0; i0 < dj; i0 += 32) arc(i0 + lane < dj, (int)(v0 + j), aj, bj + i0 + lane);
    }
    const int sd = dB <= 32 ? dB : 0;
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
    const long long cbase = __shfl_sync(TC_FULL_MASK, b - (long long)(incl - sd), src);
    const int cA = __shfl_sync(TC_FULL_MASK, dA, src);
    int before = 0;
    for (int k0 = 0; k0 < tot; k0 += 32) {
      const unsigned starts =
          __reduce_or_sync(TC_FULL_MASK, (cexcl >= k0 && cexcl < k0 + 32) ? (1u << (cexcl - k0)) : 0u);
      const int c = max(before + __popc(starts & upto) - 1, 0);
      before += __popc(starts);
      const long long base = __shfl_sync(TC_FULL_MASK, cbase, c);
      const int a = __shfl_sync(TC_FULL_MASK, cA, c);
      const int row = __shfl_sync(TC_FULL_MASK, src, c);
      const int k = k0 + lane;
      arc(k < tot, (int)(v0 + row), a, base + k);
    }
  }
  pair_holes(pb, pairs);
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    w_all += __shfl_down_sync(TC_FULL_MASK, w_all, o);
    w_min += __shfl_down_sync(TC_FULL_MASK, w_min, o);
  }
  if (lane == 0) {
    if (w_all) atomicAdd(plans + PLAN_W_ALL, w_all);
    if (w_min) atomicAdd(plans + PLAN_W_MIN, w_min);
  }
}

int tile_split_plan(trust_tc_ctx *c, const DevGraph3 &g, cudaStream_t st) {
  const size_t nt = (size_t)std::max<int64_t>(g.rowsC + 1, 1);  // targets u: rows of C
  int rc = ensure((void **)&c->d_split_cnt, &c->split_cnt_cap, sizeof(unsigned) * nt);
  if (rc) return rc;
  if ((rc = ensure((void **)&c->d_split_plans, &c->split_plans_cap, TC_PLAN_WORDS * sizeof(unsigned long long))))
    return rc;
  if ((rc = ensure((void **)&c->d_split_wsum, &c->split_wsum_cap, sizeof(unsigned long long) * nt))) return rc;
  const int blocks = arc_blocks(g.rows, c->num_sms);  // one warp per 32 rows
  const size_t slots = pair_slots(g.mB, (int64_t)blocks * 8);
  if ((rc = ensure((void **)&c->d_split_pairs, &c->split_pairs_cap, sizeof(int2) * slots))) return rc;
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_cnt, 0, sizeof(unsigned) * nt, st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_wsum, 0, sizeof(unsigned long long) * nt, st));
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_plans, 0, TC_PLAN_WORDS * sizeof(unsigned long long), st));
  tile_sched_kernel<<<blocks, 256, 0, st>>>(g.begA, g.begB, g.adjB, g.begC, g.rows, c->d_split_cnt, c->d_split_wsum,
                                            c->d_split_plans, c->d_split_pairs, slots);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaMemcpyAsync(c->h_plans, c->d_split_plans, TC_PLAN_WORDS * sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, st));
  return TRUST_TC_OK;
}

// One warp per row: any entry not below its successor marks the CSR (flag word 1).
__global__ void rows_increasing_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                                       int64_t rows, unsigned long long *flag) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int bad = 0;
  for (int64_t v = warp; v < rows; v += nwarps) {
    const long long b = tc_ld_nc(beg + v);
    const int d = (int)(tc_ld_nc(beg + v + 1) - b);
    for (int k = lane; k + 1 < d; k += 32) bad |= tc_ld_nc(adj + b + k) >= tc_ld_nc(adj + b + k + 1);
  }
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  if (lane == 0 && bad) atomicOr(flag, 1ull);
}

int rows_increasing(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t rows, cudaStream_t st,
                    bool *out) {
  int rc = ensure((void **)&c->d_split_plans, &c->split_plans_cap, TC_PLAN_WORDS * sizeof(unsigned long long));
  if (rc) return rc;
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_plans, 0, sizeof(unsigned long long), st));
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((rows + 7) / 8, (int64_t)c->num_sms * 8));
  rows_increasing_kernel<<<blocks, 256, 0, st>>>(beg, adj, rows, c->d_split_plans);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaMemcpyAsync(c->h_plans, c->d_split_plans, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  *out = c->h_plans[0] == 0;
  return TRUST_TC_OK;
}

// Build the second pass's work rows (after split_plan, whose long-row list it reuses): the
// in-list of every target, cut into chunks so one heavily targeted row spreads over many CTAs.
// Outputs live in the context.
int split_build(trust_tc_ctx *c, const int64_t *beg, const int32_t * /*adj*/, int64_t n, int64_t m, cudaStream_t st,
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
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  int64_t total = 0;
  if ((rc = scan_exclusive_i64(c->d_split_beg, c->d_split_beg, n + 1, st, &total))) return rc;
  if (total > m) return TRUST_TC_E_DEVICE;
  // chunk bases
  chunk_count_kernel<<<vb, 256, 0, st>>>(beg, c->d_split_cnt, c->d_split_wsum, c->d_split_cbase, n);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  int64_t nchunks = 0;
  if ((rc = scan_exclusive_i64(c->d_split_cbase, c->d_split_cbase, n + 1, st, &nchunks))) return rc;
  if (nchunks > max_chunks) return TRUST_TC_E_DEVICE;
  // scatter the sources; the in-degree counts (read by chunk_count_kernel above) become the cursors
  TC_CUDA_TRY(cudaMemsetAsync(c->d_split_cnt, 0, sizeof(unsigned) * (size_t)(n + 1), st));
  split_fill_kernel<<<arc_blocks(m, c->num_sms), 256, 0, st>>>(c->d_split_pairs, c->d_split_plans + PLAN_NPAIRS,
                                                               c->d_split_beg, c->d_split_cnt, c->d_split_adj);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  chunk_fill_kernel<<<vb, 256, 0, st>>>(c->d_split_cbase, c->d_split_beg, n, total, nchunks, c->d_split_cbeg,
                                        c->d_split_rowmap);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  out->beg = c->d_split_cbeg;
  out->adj = c->d_split_adj;
  out->rowmap = c->d_split_rowmap;
  out->rows = nchunks;
  out->m = total;
  return TRUST_TC_OK;
}

// ---- heaviest-first queue order ------------------------------------------------------------------
// A counting sort of the warp, CTA and huge lists (adjacent in the list buffer, in that order) by
// predicted cost, descending, in buckets of 1/8 log2 cycle.  The order inside a bucket is
// arbitrary: a work queue only needs its long rows first.
constexpr int TC_LPT_BUCKETS = 256;
constexpr int TC_LPT_KEYS = 3 * TC_LPT_BUCKETS;  // (class, bucket)

struct LptRange {
  int lo, cta, huge, hi;  // list indices: [lo, cta) warp, [cta, huge) CTA, [huge, hi) huge
};

__device__ __forceinline__ int lpt_key(const LptRange &r, int i, float y) {
  const int c = i < r.cta ? 0 : (i < r.huge ? 1 : 2);
  const int q = (int)(fminf(fmaxf(y, 0.f), 31.99f) * 8.f);  // 0..255
  return c * TC_LPT_BUCKETS + (TC_LPT_BUCKETS - 1 - q);     // larger prediction first
}

__global__ void lpt_hist_kernel(const int *__restrict__ lists, LptRange r, const float *__restrict__ pred,
                                unsigned *__restrict__ hist) {
  __shared__ unsigned h[TC_LPT_KEYS];
  for (int i = threadIdx.x; i < TC_LPT_KEYS; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (int i = r.lo + blockIdx.x * blockDim.x + threadIdx.x; i < r.hi; i += gridDim.x * blockDim.x)
    atomicAdd(&h[lpt_key(r, i, pred[lists[i]])], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < TC_LPT_KEYS; i += blockDim.x)
    if (h[i]) atomicAdd(hist + i, h[i]);
}

// Every CTA (256 threads) scans the histogram itself, then places its items through per-key
// cursors (one atomic per key and warp).  out[] is indexed from r.lo.
__global__ void __launch_bounds__(256) lpt_scatter_kernel(const int *__restrict__ lists, LptRange r,
                                                          const float *__restrict__ pred,
                                                          const unsigned *__restrict__ hist,
                                                          unsigned *__restrict__ cursor, int *__restrict__ out) {
  __shared__ unsigned base[TC_LPT_KEYS];
  __shared__ unsigned wsum[8];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int cls_start[3] = {0, r.cta - r.lo, r.huge - r.lo};
  for (int c = 0; c < 3; ++c) {  // exclusive scan of class c's buckets, thread t owns bucket t
    const unsigned x = hist[c * TC_LPT_BUCKETS + t];
    unsigned incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(TC_FULL_MASK, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    unsigned before = 0;
    for (int k = 0; k < w; ++k) before += wsum[k];
    base[c * TC_LPT_BUCKETS + t] = (unsigned)cls_start[c] + before + incl - x;
    __syncthreads();
  }
  for (int i0 = r.lo + blockIdx.x * blockDim.x; i0 < r.hi; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + t;
    int key = -1, v = 0;
    if (i < r.hi) {
      v = lists[i];
      key = lpt_key(r, i, pred[v]);
    }
    const unsigned peers = __match_any_sync(TC_FULL_MASK, key);
    const int leader = __ffs(peers) - 1;
    unsigned at = 0;
    if (key >= 0 && lane == leader) at = atomicAdd(cursor + key, (unsigned)__popc(peers));
    at = __shfl_sync(TC_FULL_MASK, at, leader);
    if (key >= 0) out[base[key] + at + __popc(peers & tc_lanemask_lt())] = v;
  }
}

int lpt_sort(trust_tc_ctx *c, int *lists, const int *off, const int *counts, const float *pred, cudaStream_t st) {
  LptRange r;
  r.lo = off[TC_CLASS_WARP];
  r.cta = off[TC_CLASS_CTA];
  r.huge = off[TC_CLASS_HUGE];
  r.hi = off[TC_CLASS_HUGE] + counts[TC_CLASS_HUGE];
  const int total = r.hi - r.lo;
  if (total < 2) return TRUST_TC_OK;
  // scratch: histogram and cursors (2 x TC_LPT_KEYS u32), then the sorted copy
  const size_t bytes = sizeof(unsigned) * (2 * (size_t)TC_LPT_KEYS + (size_t)total);
  int rc = ensure((void **)&c->d_sort, &c->sort_cap, bytes);
  if (rc) return rc;
  unsigned *hist = reinterpret_cast<unsigned *>(c->d_sort);
  unsigned *cursor = hist + TC_LPT_KEYS;
  int *out = reinterpret_cast<int *>(cursor + TC_LPT_KEYS);
  TC_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(unsigned) * 2 * TC_LPT_KEYS, st));
  const int blocks = std::max(1, std::min((total + 255) / 256, c->num_sms * 2));
  lpt_hist_kernel<<<blocks, 256, 0, st>>>(lists, r, pred, hist);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  lpt_scatter_kernel<<<blocks, 256, 0, st>>>(lists, r, pred, hist, cursor, out);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  TC_CUDA_TRY(cudaMemcpyAsync(lists + r.lo, out, sizeof(int) * (size_t)total, cudaMemcpyDeviceToDevice, st));
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
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

}  // namespace tc

// tc_count.cu — the vertex-centric hash build + probe counting kernels for sm_103a.
//
// Replaces dynamic_assign (Without-graph-partition/TC.cu:230-600) and its partitioned twin
// (With-graph-partition/TC.cu:630-973).  Same method — a hash table of N+(v) per source vertex,
// probed with every w in N+(u) for u in N+(v) — with a different schedule:
//   * a classification pass sorts vertices into size classes by out-degree (the reference's
//     USE_CTA / USE_WARP thresholds, TC.cu:19-20, generalised to sub-warp groups);
//   * one persistent kernel drains the class queues largest-first with atomic chunk claims
//     (the reference's G_INDEX work stealing, TC.cu:405-422 and :560-577);
//   * the probe work of a vertex is flattened over lanes with a shuffle prefix scan and a
//     shuffle binary search, so no lane re-walks neighbour lists (the reference re-reads
//     adj/beg for every skipped list, TC.cu:342-349 and :522-529);
//   * tables are open-addressing sets sized 2x the list, so nothing is ever dropped (the
//     reference drops the 101st entry of a bucket, TC.cu:299).
// The counted quantity is documented in include/trust_tc.h.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "tc_count.h"

namespace tc {

// ------------------------------------------------------------------------------------------
// hash-set primitives (open addressing, linear probing, -1 = empty; ids are validated >= 0)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ bool set_insert(int *tab, int log2, int key) {
  const unsigned mask = (1u << log2) - 1u;
  unsigned h = tc_hash((unsigned)key, log2);
  for (unsigned it = 0; it <= mask; ++it) {
    int prev = atomicCAS(tab + h, -1, key);
    if (prev == -1 || prev == key) return true;
    h = (h + 1u) & mask;
  }
  return false;
}

__device__ __forceinline__ int set_probe(const int *tab, int log2, int key) {
  const unsigned mask = (1u << log2) - 1u;
  unsigned h = tc_hash((unsigned)key, log2);
  for (unsigned it = 0; it <= mask; ++it) {
    int x = tab[h];
    if (x == key) return 1;
    if (x < 0) return 0;
    h = (h + 1u) & mask;
  }
  return 0;
}

template <int G>
__device__ __forceinline__ int group_scan_incl(int x, int glane) {
#pragma unroll
  for (int off = 1; off < G; off <<= 1) {
    int y = __shfl_up_sync(TC_FULL_MASK, x, off, G);
    if (glane >= off) x += y;
  }
  return x;
}

// Number of lanes of the G-lane group whose (non-decreasing) `incl` is <= k.  All 32 lanes
// of the warp must call it; every lane may ask about a different k.
template <int G>
__device__ __forceinline__ int group_count_le(int incl, int k) {
  int j = 0;
#pragma unroll
  for (int step = G / 2; step >= 1; step >>= 1) {
    int t = __shfl_sync(TC_FULL_MASK, incl, j + step - 1, G);
    if (t <= k) j += step;
  }
  return j;
}

// Membership in the source row N+(v), held in registers of every lane of the group (rows of at
// most G <= 8 entries; lanes past the row hold -1, which no id equals).
template <int G>
struct RegSet {
  int key[G];
  __device__ __forceinline__ void load(int mine) {
#pragma unroll
    for (int i = 0; i < G; ++i) key[i] = __shfl_sync(TC_FULL_MASK, mine, i, G);
  }
  __device__ __forceinline__ int has(int w) const {
    bool h = false;
#pragma unroll
    for (int i = 0; i < G; ++i) h |= key[i] == w;
    return h;
  }
};

// Membership in an open-addressing table (shared or global memory).
struct HashSet {
  const int *tab;
  int log2;
  __device__ __forceinline__ int has(int w) const { return set_probe(tab, log2, w); }
};

constexpr int TC_UNROLL = 2;  // independent neighbour-row loads in flight per lane

// Probe every wedge of the arcs held one per lane of a G-lane group against `set`.
// Lane state: the arc's target row start `s` (int: m < 2^31) and length `dd` (0 if idle).
// Rows of at least G entries are walked by the whole group, G consecutive entries per step
// (coalesced, no index search); shorter rows are flattened with a shuffle prefix scan and each
// lane finds its row by a shuffle binary search.  All 32 lanes call it.
template <int G, class Set>
__device__ __forceinline__ void probe_arcs(const int32_t *__restrict__ adjC, int s, int dd, int glane,
                                           const Set &set, unsigned long long &hits,
                                           unsigned long long &wedges) {
  constexpr int U = TC_UNROLL;
  wedges += (unsigned)dd;
  const int lane = threadIdx.x & 31;
  const int gbase = lane & ~(G - 1);
  const unsigned gbits = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
  unsigned mine = (__ballot_sync(TC_FULL_MASK, dd >= G) >> gbase) & gbits;
  // long rows: one row at a time per group
  while (__any_sync(TC_FULL_MASK, mine != 0)) {
    const bool have = mine != 0;
    const int j = have ? __ffs(mine) - 1 : 0;
    mine &= mine - 1;
    const int sj = __shfl_sync(TC_FULL_MASK, s, j, G);
    int dj = __shfl_sync(TC_FULL_MASK, dd, j, G);
    if (!have) dj = 0;
    for (int k = glane; k < dj; k += G * U) {
      int w[U];
#pragma unroll
      for (int r = 0; r < U; ++r) w[r] = k + r * G < dj ? tc_ld_nc(adjC + sj + k + r * G) : -1;
#pragma unroll
      for (int r = 0; r < U; ++r)
        if (w[r] >= 0) hits += set.has(w[r]);
    }
  }
  // short rows: flattened over the group's lanes
  const int sd = dd < G ? dd : 0;
  const int incl = group_scan_incl<G>(sd, glane);
  const int tot = __shfl_sync(TC_FULL_MASK, incl, G - 1, G);
  const int base = s - (incl - sd);
  const int totmax = __reduce_max_sync(TC_FULL_MASK, tot);
  for (int k0 = 0; k0 < totmax; k0 += G * U) {
    int w[U];
#pragma unroll
    for (int r = 0; r < U; ++r) {
      const int k = k0 + r * G + glane;
      const int j = group_count_le<G>(incl, k);
      const int bj = __shfl_sync(TC_FULL_MASK, base, j, G);
      w[r] = k < tot ? tc_ld_nc(adjC + bj + k) : -1;
    }
#pragma unroll
    for (int r = 0; r < U; ++r)
      if (w[r] >= 0) hits += set.has(w[r]);
  }
}

// ------------------------------------------------------------------------------------------
// validation / classification
// ------------------------------------------------------------------------------------------
__global__ void check_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj,
                             int64_t rows, int64_t m, int64_t id_bound, int check_ids,
                             TcControl *ctl) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int bad = 0;
  int dmax = 0;
  for (int64_t v = tid; v < rows; v += stride) {
    long long b = tc_ld_nc(beg + v), e = tc_ld_nc(beg + v + 1);
    if (e < b || b < 0 || e > m) {
      bad |= TC_DEV_BAD_OFFSETS;
    } else if (e - b >= (1ll << 26)) {
      bad |= TC_DEV_TOO_LARGE;
    } else {
      dmax = max(dmax, (int)(e - b));
    }
  }
  if (tid == 0) {
    if (tc_ld_nc(beg) != 0 || tc_ld_nc(beg + rows) != m) bad |= TC_DEV_BAD_OFFSETS;
  }
  if (check_ids) {
    for (int64_t i = tid; i < m; i += stride) {
      int x = tc_ld_nc(adj + i);
      if (x < 0 || (int64_t)x >= id_bound) bad |= TC_DEV_BAD_IDS;
    }
  }
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  dmax = __reduce_max_sync(TC_FULL_MASK, dmax);
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(&ctl->status, bad);
    atomicMax(&ctl->max_out_degree, dmax);
  }
}

__device__ __forceinline__ int classify(int dA, int dB, int min_deg, int warp_max, int cta_max) {
  if (dA < min_deg || dB < min_deg) return TC_CLASS_SKIP;
  int d = max(dA, dB);
  if (d <= 4) return TC_CLASS_G4;
  if (d <= 8) return TC_CLASS_G8;
  if (d <= 16) return TC_CLASS_G16;
  if (d <= 32) return TC_CLASS_G32;
  if (d <= warp_max) return TC_CLASS_WARP;
  if (d <= cta_max) return TC_CLASS_CTA;
  return TC_CLASS_HUGE;
}

// pass 0: histogram of classes.  pass 1: scatter vertex ids into per-class lists.
template <int PASS>
__global__ void class_kernel(const int64_t *__restrict__ begA, const int64_t *__restrict__ begB,
                             int64_t rows, int min_deg, int warp_max, int cta_max,
                             TcControl *ctl, int *__restrict__ lists, ListOffsets off) {
  __shared__ int s_hist[TC_NUM_CLASSES];
  __shared__ int s_base[TC_NUM_CLASSES];
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < rows; base += stride) {
    if (threadIdx.x < TC_NUM_CLASSES) s_hist[threadIdx.x] = 0;
    __syncthreads();
    int64_t v = base + threadIdx.x;
    int c = -1;
    if (v < rows) {
      int dA = (int)(tc_ld_nc(begA + v + 1) - tc_ld_nc(begA + v));
      int dB = (begB == begA) ? dA : (int)(tc_ld_nc(begB + v + 1) - tc_ld_nc(begB + v));
      c = classify(dA, dB, min_deg, warp_max, cta_max);
    }
    // warp-aggregated block histogram, then one global reservation per class per block
    unsigned peers = __match_any_sync(TC_FULL_MASK, c);
    int rank = __popc(peers & tc_lanemask_lt());
    int wbase = 0;
    if (c >= 0 && rank == 0) wbase = atomicAdd(&s_hist[c], __popc(peers));
    int leader = __ffs(peers) - 1;
    wbase = __shfl_sync(TC_FULL_MASK, wbase, leader);
    __syncthreads();
    if (PASS == 0) {
      if (threadIdx.x < TC_NUM_CLASSES && s_hist[threadIdx.x])
        atomicAdd(&ctl->class_count[threadIdx.x], s_hist[threadIdx.x]);
    } else {
      if (threadIdx.x < TC_NUM_CLASSES && s_hist[threadIdx.x])
        s_base[threadIdx.x] = atomicAdd(&ctl->class_cursor[threadIdx.x], s_hist[threadIdx.x]);
      __syncthreads();
      if (c > TC_CLASS_SKIP) lists[off.off[c] + s_base[c] + wbase + rank] = (int)v;
    }
    __syncthreads();
  }
  (void)lane;
}

// ------------------------------------------------------------------------------------------
// the persistent counting kernel
// ------------------------------------------------------------------------------------------
struct BlockShared {
  unsigned long long count;
  unsigned long long wedges;
  int item;
  int next_batch;
};

__device__ __forceinline__ int ceil_log2_table(int d) {
  // smallest power of two >= 2d, at least 64 slots
  int need = max(2 * d, 64);
  return 32 - __clz(need - 1);
}

// Row start and length of v (int: m < 2^31 is enforced on the host).
__device__ __forceinline__ void row_of(const int64_t *__restrict__ beg, int v, int &b, int &d) {
  const long long lo = tc_ld_nc(beg + v), hi = tc_ld_nc(beg + v + 1);
  b = (int)lo;
  d = (int)(hi - lo);
}

// One vertex handled by a whole CTA.  `tab` is shared (CTA class) or global (huge class).
// Warps claim 32-arc batches of the vertex from a shared counter.
template <bool SAME>
__device__ void cta_vertex(const CountArgs &p, int v, int *tab, BlockShared &bs, unsigned long long &hits,
                           unsigned long long &wedges) {
  const int lane = threadIdx.x & 31;
  int bA, dA, bB, dB;
  row_of(p.begA, v, bA, dA);
  if (SAME) { bB = bA; dB = dA; } else { row_of(p.begB, v, bB, dB); }
  const int log2 = ceil_log2_table(dA);
  const int T = 1 << log2;
  for (int i = threadIdx.x; i < T; i += blockDim.x) tab[i] = -1;
  if (threadIdx.x == 0) bs.next_batch = 0;
  __syncthreads();
  bool ok = true;
  for (int i = threadIdx.x; i < dA; i += blockDim.x) ok &= set_insert(tab, log2, tc_ld_nc(p.adjA + bA + i));
  if (!ok) atomicOr(&p.ctl->status, TC_DEV_TABLE_FULL);
  __syncthreads();
  const HashSet set{tab, log2};
  const int nbatch = (dB + 31) >> 5;
  for (;;) {
    int bt = 0;
    if (lane == 0) bt = atomicAdd(&bs.next_batch, 1);
    bt = __shfl_sync(TC_FULL_MASK, bt, 0);
    if (bt >= nbatch) break;
    const int i = (bt << 5) + lane;
    int s = 0, dd = 0;
    if (i < dB) row_of(p.begC, tc_ld_nc(p.adjB + bB + i), s, dd);
    probe_arcs<32>(p.adjC, s, dd, lane, set, hits, wedges);
  }
  __syncthreads();
}

// One vertex per warp, 32 < out-degree <= warp_max: several 32-arc rounds on a warp table.
template <bool SAME>
__device__ __forceinline__ void warp_vertex(const CountArgs &p, int v, int *warp_tab, unsigned long long &hits,
                                            unsigned long long &wedges) {
  const int lane = threadIdx.x & 31;
  int bA, dA, bB, dB;
  row_of(p.begA, v, bA, dA);
  if (SAME) { bB = bA; dB = dA; } else { row_of(p.begB, v, bB, dB); }
  const int log2 = ceil_log2_table(dA);
  const int T = 1 << log2;
  for (int i = lane; i < T; i += 32) warp_tab[i] = -1;
  __syncwarp();
  bool ok = true;
  for (int i = lane; i < dA; i += 32) ok &= set_insert(warp_tab, log2, tc_ld_nc(p.adjA + bA + i));
  if (!ok) atomicOr(&p.ctl->status, TC_DEV_TABLE_FULL);
  __syncwarp();
  const HashSet set{warp_tab, log2};
  for (int a0 = 0; a0 < dB; a0 += 32) {
    const int i = a0 + lane;
    int s = 0, dd = 0;
    if (i < dB) row_of(p.begC, tc_ld_nc(p.adjB + bB + i), s, dd);
    probe_arcs<32>(p.adjC, s, dd, lane, set, hits, wedges);
  }
  __syncwarp();
}

// One vertex per G-lane group (G = 4, 8, 16, 32), out-degrees <= G.  The vertex's row bounds
// (bA, dA) were loaded one step ahead by the caller.
template <int G, bool SAME>
__device__ __forceinline__ void group_vertex(const CountArgs &p, int v, int bA, int dA, int *grp_tab,
                                             unsigned long long &hits, unsigned long long &wedges) {
  const int glane = threadIdx.x & (G - 1);
  int bB = bA, dB = dA;
  if (!SAME && v >= 0) row_of(p.begB, v, bB, dB);
  const int uA = glane < dA ? tc_ld_nc(p.adjA + bA + glane) : -1;
  const int uB = SAME ? uA : (glane < dB ? tc_ld_nc(p.adjB + bB + glane) : -1);
  int s = 0, dd = 0;
  if (uB >= 0) row_of(p.begC, uB, s, dd);
  if constexpr (G <= 8) {
    RegSet<G> set;
    set.load(uA);
    probe_arcs<G>(p.adjC, s, dd, glane, set, hits, wedges);
  } else {
    constexpr int LOG2 = (G == 16 ? 4 : 5) + 2;  // 4G slots per group
#pragma unroll
    for (int i = glane; i < 4 * G; i += G) grp_tab[i] = -1;
    __syncwarp();
    if (uA >= 0) set_insert(grp_tab, LOG2, uA);
    __syncwarp();
    probe_arcs<G>(p.adjC, s, dd, glane, HashSet{grp_tab, LOG2}, hits, wedges);
    __syncwarp();
  }
}

// Drain one group class.  Each warp claims `chunk` steps of 32/G vertices; the next step's row
// bounds are loaded while the current step is probed.
template <int G, bool SAME>
__device__ void drain_group_class(const CountArgs &p, int c, int *warp_tab, unsigned long long &hits,
                                  unsigned long long &wedges) {
  constexpr int GPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  int *grp_tab = warp_tab + g * (4 * G);
  const int n_items = p.ctl->class_count[c];
  const int *list = p.lists + p.off.off[c];
  const int claim = p.chunk * GPW;
  for (;;) {
    int t0 = 0;
    if (lane == 0) t0 = atomicAdd(&p.ctl->class_next[c], claim);
    t0 = __shfl_sync(TC_FULL_MASK, t0, 0);
    if (t0 >= n_items) break;
    const int t1 = min(t0 + claim, n_items);
    int v = t0 + g < t1 ? list[t0 + g] : -1;
    int vn = t0 + GPW + g < t1 ? list[t0 + GPW + g] : -1;
    int b = 0, d = 0;
    if (v >= 0) row_of(p.begA, v, b, d);
    for (int t = t0; t < t1; t += GPW) {
      // prefetch: row bounds of the next step, list entry of the one after
      int bn = 0, dn = 0;
      if (vn >= 0) row_of(p.begA, vn, bn, dn);
      const int item2 = t + 2 * GPW + g;
      const int vnn = item2 < t1 ? list[item2] : -1;
      group_vertex<G, SAME>(p, v, b, d, grp_tab, hits, wedges);
      v = vn;
      vn = vnn;
      b = bn;
      d = dn;
    }
  }
}

// Two register budgets: up to 1024 threads per CTA (reference launch shape), or <= 256 threads
// with at least TC_MIN_CTAS_256 CTAs resident per SM (the default shape).
constexpr int TC_MIN_CTAS_256 = 5;

template <bool SAME, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) count_kernel(CountArgs p) {
  extern __shared__ int smem[];
  __shared__ BlockShared bs;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) bs.count = bs.wedges = 0;
  unsigned long long hits = 0, wedges = 0;

  // Phase A: CTA-granularity vertices, largest class first.
  for (int c = TC_CLASS_HUGE; c >= TC_CLASS_CTA; --c) {
    const int n_items = p.ctl->class_count[c];
    if (n_items == 0) continue;
    if (c == TC_CLASS_HUGE && (int)blockIdx.x >= p.huge_blocks) continue;
    const int *list = p.lists + p.off.off[c];
    int *tab = (c == TC_CLASS_HUGE) ? p.huge_tables + (size_t)blockIdx.x * ((size_t)1 << p.huge_log2)
                                    : smem;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) bs.item = atomicAdd(&p.ctl->class_next[c], 1);
      __syncthreads();
      const int t = bs.item;
      if (t >= n_items) break;
      cta_vertex<SAME>(p, list[t], tab, bs, hits, wedges);
    }
  }
  __syncthreads();

  // Phase B: warp and sub-warp granularity.
  int *warp_tab = smem + warp * p.warp_slots;
  {
    const int c = TC_CLASS_WARP;
    const int n_items = p.ctl->class_count[c];
    const int *list = p.lists + p.off.off[c];
    for (;;) {
      int t0 = 0;
      if (lane == 0) t0 = atomicAdd(&p.ctl->class_next[c], p.chunk);
      t0 = __shfl_sync(TC_FULL_MASK, t0, 0);
      if (t0 >= n_items) break;
      const int t1 = min(t0 + p.chunk, n_items);
      for (int t = t0; t < t1; ++t) warp_vertex<SAME>(p, list[t], warp_tab, hits, wedges);
    }
  }
  drain_group_class<32, SAME>(p, TC_CLASS_G32, warp_tab, hits, wedges);
  drain_group_class<16, SAME>(p, TC_CLASS_G16, warp_tab, hits, wedges);
  drain_group_class<8, SAME>(p, TC_CLASS_G8, warp_tab, hits, wedges);
  drain_group_class<4, SAME>(p, TC_CLASS_G4, warp_tab, hits, wedges);

  // Reduction: warp shuffle -> shared u64 -> one global u64 atomic per CTA
  // (the reference does per-thread shared atomics, Without-graph-partition/TC.cu:586-599).
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    hits += __shfl_down_sync(TC_FULL_MASK, hits, off);
    wedges += __shfl_down_sync(TC_FULL_MASK, wedges, off);
  }
  if (lane == 0 && hits) atomicAdd(&bs.count, hits);
  if (lane == 0 && wedges) atomicAdd(&bs.wedges, wedges);
  __syncthreads();
  if (threadIdx.x == 0 && bs.count) atomicAdd(&p.ctl->count, bs.count);
  if (threadIdx.x == 0 && bs.wedges) atomicAdd(&p.ctl->wedges, bs.wedges);
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
int launch_check(const int64_t *beg, const int32_t *adj, int64_t rows, int64_t m, int64_t id_bound,
                 int check_ids, TcControl *ctl, int num_sms, cudaStream_t st) {
  int64_t work = std::max<int64_t>(rows, check_ids ? m : 0);
  int blocks = (int)std::min<int64_t>((work + 255) / 256, (int64_t)num_sms * 8);
  blocks = std::max(blocks, 1);
  check_kernel<<<blocks, 256, 0, st>>>(beg, adj, rows, m, id_bound, check_ids, ctl);
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

int launch_classify(int pass, const int64_t *begA, const int64_t *begB, int64_t rows, int min_deg,
                    int warp_max, int cta_max, TcControl *ctl, int *lists, const ListOffsets &off,
                    int num_sms, cudaStream_t st) {
  int blocks = (int)std::min<int64_t>((rows + 255) / 256, (int64_t)num_sms * 8);
  blocks = std::max(blocks, 1);
  if (pass == 0)
    class_kernel<0><<<blocks, 256, 0, st>>>(begA, begB, rows, min_deg, warp_max, cta_max, ctl, lists, off);
  else
    class_kernel<1><<<blocks, 256, 0, st>>>(begA, begB, rows, min_deg, warp_max, cta_max, ctl, lists, off);
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

template <bool SAME, int MAXT, int MINB>
static cudaError_t occupancy_of(int threads, size_t smem_bytes, int *blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(count_kernel<SAME, MAXT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_bytes);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, count_kernel<SAME, MAXT, MINB>, threads,
                                                      smem_bytes);
  return e;
}

int count_kernel_occupancy(bool same, int threads, size_t smem_bytes, int *blocks_per_sm) {
  cudaError_t e;
  if (threads <= 256)
    e = same ? occupancy_of<true, 256, TC_MIN_CTAS_256>(threads, smem_bytes, blocks_per_sm)
             : occupancy_of<false, 256, TC_MIN_CTAS_256>(threads, smem_bytes, blocks_per_sm);
  else
    e = same ? occupancy_of<true, 1024, 1>(threads, smem_bytes, blocks_per_sm)
             : occupancy_of<false, 1024, 1>(threads, smem_bytes, blocks_per_sm);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

int launch_count(bool same, const CountArgs &a, int blocks, int threads, size_t smem_bytes,
                 cudaStream_t st) {
  if (threads <= 256) {
    if (same)
      count_kernel<true, 256, TC_MIN_CTAS_256><<<blocks, threads, smem_bytes, st>>>(a);
    else
      count_kernel<false, 256, TC_MIN_CTAS_256><<<blocks, threads, smem_bytes, st>>>(a);
  } else {
    if (same)
      count_kernel<true, 1024, 1><<<blocks, threads, smem_bytes, st>>>(a);
    else
      count_kernel<false, 1024, 1><<<blocks, threads, smem_bytes, st>>>(a);
  }
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

}  // namespace tc

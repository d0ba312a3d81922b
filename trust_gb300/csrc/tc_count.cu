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
#include <map>
#include <mutex>
#include <tuple>

#include <cooperative_groups.h>

#include "tc_count.h"

namespace tc {

// ------------------------------------------------------------------------------------------
// hash-set primitives (open addressing, linear probing, -1 = empty; ids are validated >= 0)
// ------------------------------------------------------------------------------------------
// Tables are 2^log2 int slots (log2 >= 6) read as buckets of four (16-byte loads).  A key's home
// is the first slot of bucket hash(key); insertion takes the first free slot from there on
// (linear probing over slots), so a lookup that finds an empty slot in a bucket without the key
// can stop: the key would have been placed there.
__device__ __forceinline__ bool set_insert(int *tab, int log2, int key) {
  const unsigned mask = (1u << log2) - 1u;
  unsigned h = tc_hash((unsigned)key, log2 - 2) << 2;
  for (unsigned it = 0; it <= mask; ++it) {
    int prev = atomicCAS(tab + h, -1, key);
    if (prev == -1 || prev == key) return true;
    h = (h + 1u) & mask;
  }
  return false;
}

__device__ __forceinline__ int set_probe(const int *tab, int log2, int key) {
  const unsigned bmask = (1u << (log2 - 2)) - 1u;
  unsigned b = tc_hash((unsigned)key, log2 - 2);
  for (unsigned it = 0; it <= bmask; ++it) {
    const int4 q = *reinterpret_cast<const int4 *>(tab + (b << 2));
    if (q.x == key || q.y == key || q.z == key || q.w == key) return 1;
    if ((q.x | q.y | q.z | q.w) < 0) return 0;  // an empty slot (-1) ends the search
    b = (b + 1u) & bmask;
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

// Membership in an open-addressing table (shared or global memory).
struct HashSet {
  const int *tab;
  int log2;
  __device__ __forceinline__ int has(int w) const { return set_probe(tab, log2, w); }
};

// Quotient tables (CTA-class rows, shared memory): keys are ids below 2^kb (kb <= 26).  The map
// h(k) = k * M mod 2^kb (M odd) is a bijection of [0, 2^kb), so a key is identified by the pair
// (home bucket = top bb bits of h, remainder = low kb - bb bits) and a slot stores the remainder
// alone: 16-bit slots (remainders <= 15 bits, 0xFFFF = empty), 8 per 16-byte bucket.  In the bytes
// of a 32-bit table at half load the same row fills a quarter of the slots, so a home bucket is
// full with probability about 0.1 % (2 keys per 8 slots on average) and a lookup is one 16-byte
// load: no warp-divergent further rounds for the lanes whose bucket overflowed, which in 4-slot
// buckets at half load hit nearly every warp (about a third of the count's time on R-MAT 26).
// A remainder means something only in its home bucket, so a key whose home bucket is full goes,
// whole, to a short overflow list after the buckets; a lookup reads that list only when its home
// bucket is full.  Slots of a bucket fill in order (an insert takes the first free slot), so an
// empty last slot means the bucket was never full.  If the list itself fills (not expected), the
// row is rebuilt as a 32-bit table.
constexpr unsigned TC_Q16_MULT = 0x9E3779B1u;
constexpr int TC_Q16_MAX_KEY_BITS = 26;  // 2^(kb - 15) buckets must fit the CTA table's bytes
constexpr int TC_Q16_OVERFLOW = 128;     // overflow list entries (512 bytes after the buckets)

__device__ __forceinline__ unsigned q16_haszero(unsigned x) {  // some 16-bit half of x is 0
  return (x - 0x00010001u) & ~x & 0x80008000u;
}

struct Q16Set {
  const unsigned short *tab;
  int bb;          // log2 buckets
  int kb;          // key bits
  const int *ov;   // keys whose home bucket was full
  int n_ov;
  __device__ __forceinline__ int has(int key) const {
    const unsigned h = ((unsigned)key * TC_Q16_MULT) & ((1u << kb) - 1u);
    const int rb = kb - bb;
    const unsigned b = h >> rb;
    const unsigned r = h & ((1u << rb) - 1u);
    const unsigned rr = r | (r << 16);
    const uint4 q = *reinterpret_cast<const uint4 *>(tab + 8 * b);
    if (q16_haszero(q.x ^ rr) | q16_haszero(q.y ^ rr) | q16_haszero(q.z ^ rr) | q16_haszero(q.w ^ rr)) return 1;
    if (q.w >= 0xFFFF0000u) return 0;  // last slot empty: the home bucket was never full
    for (int i = 0; i < n_ov; ++i)
      if (ov[i] == key) return 1;
    return 0;
  }
};

// Insert into the key's home bucket; false when that bucket is full (the caller lists the key).
__device__ __forceinline__ bool q16_insert(unsigned short *tab, int bb, int kb, int key) {
  const unsigned h = ((unsigned)key * TC_Q16_MULT) & ((1u << kb) - 1u);
  const int rb = kb - bb;
  const unsigned b = h >> rb;
  const unsigned short r = (unsigned short)(h & ((1u << rb) - 1u));
#pragma unroll 1
  for (int j = 0; j < 8; ++j) {
    const unsigned short prev = atomicCAS(tab + 8 * b + j, (unsigned short)0xFFFF, r);
    if (prev == 0xFFFF || prev == r) return true;
  }
  return false;
}

// log2 buckets of a row of d keys in a quotient table: at least d/2 buckets (a quarter of the
// slots used) and enough buckets that remainders fit 15 bits; -1 when the buckets and the
// overflow list exceed the bytes available (the row takes a 32-bit table instead).
__device__ __forceinline__ int q16_log2_buckets(int d, int kb, int table_bytes) {
  if (kb <= 0 || kb > TC_Q16_MAX_KEY_BITS) return -1;
  int bb = 0;
  while ((1 << (bb + 1)) < d) ++bb;  // 2^(bb+1) >= d
  bb = max(bb, kb - 15);
  bb = min(bb, kb);
  return (16 << bb) + 4 * TC_Q16_OVERFLOW <= table_bytes ? bb : -1;
}

constexpr int TC_UNROLL = 4;  // independent neighbour-row loads in flight per lane

// Probe every wedge of the arcs held one per lane of a G-lane group against `set`.
// Lane state: the arc's target row start `s` (int: m < 2^31) and length `dd` (0 if idle).
// Rows of at least LONG entries are walked by the whole group, G consecutive entries per load
// (coalesced, no index search), with the next U loads issued before the current U are probed;
// shorter rows are flattened with a shuffle prefix scan and each lane finds its row by a shuffle
// binary search.  All 32 lanes call it.
template <int G, int LONG, class Set>
__device__ __forceinline__ void probe_arcs(const int32_t *__restrict__ adjC, int s, int dd, int glane,
                                           const Set &set, unsigned long long &hits,
                                           unsigned long long &wedges) {
  constexpr int U = TC_UNROLL;
  wedges += (unsigned)dd;
  const int lane = threadIdx.x & 31;
  const int gbase = lane & ~(G - 1);
  const unsigned gbits = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
  unsigned mine = (__ballot_sync(TC_FULL_MASK, dd >= LONG) >> gbase) & gbits;
  // long rows: one row at a time per group
  while (__any_sync(TC_FULL_MASK, mine != 0)) {
    const bool have = mine != 0;
    const int j = have ? __ffs(mine) - 1 : 0;
    mine &= mine - 1;
    const int sj = __shfl_sync(TC_FULL_MASK, s, j, G);
    int dj = __shfl_sync(TC_FULL_MASK, dd, j, G);
    if (!have) dj = 0;
    const int32_t *row = adjC + sj;
    int w[U];
#pragma unroll
    for (int r = 0; r < U; ++r) w[r] = glane + r * G < dj ? tc_ld_nc(row + glane + r * G) : -1;
    for (int k = glane; k < dj; k += G * U) {
      const int kn = k + G * U;
      int wn[U];
#pragma unroll
      for (int r = 0; r < U; ++r) wn[r] = kn + r * G < dj ? tc_ld_nc(row + kn + r * G) : -1;
#pragma unroll
      for (int r = 0; r < U; ++r)
        if (w[r] >= 0) hits += set.has(w[r]);
#pragma unroll
      for (int r = 0; r < U; ++r) w[r] = wn[r];
    }
  }
  // short rows: flattened over the group's lanes
  const int sd = dd < LONG ? dd : 0;
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

// Rows at least this long are walked row by row by a group of G lanes.
template <int G>
struct LongRow {
  static constexpr int value = G;
};

// Position (0..31) of the n-th (0-based) set bit of mask; mask must have more than n set bits.
__device__ __forceinline__ int nth_set_bit(unsigned mask, int n) {
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

// Membership of w in the source row of group g of this warp.  G <= 8: the rows are staged in
// shared memory as G keys per group (-1 past the row), read with 16-byte loads.  G >= 16: each
// group owns a 4G-slot hash table.
template <int G>
__device__ __forceinline__ int group_has(const int *wtab, int g, int w) {
  if constexpr (G == 4) {
    const int4 q = *reinterpret_cast<const int4 *>(wtab + 4 * g);
    return (q.x == w) | (q.y == w) | (q.z == w) | (q.w == w);
  } else if constexpr (G == 8) {
    const int4 q0 = *reinterpret_cast<const int4 *>(wtab + 8 * g);
    const int4 q1 = *reinterpret_cast<const int4 *>(wtab + 8 * g + 4);
    return (q0.x == w) | (q0.y == w) | (q0.z == w) | (q0.w == w) | (q1.x == w) | (q1.y == w) | (q1.z == w) |
           (q1.w == w);
  } else {
    constexpr int LOG2 = (G == 16 ? 4 : 5) + 2;
    return set_probe(wtab + g * (4 * G), LOG2, w);
  }
}

// Membership of w in a row of at most G keys held in registers (-1 past the row; w >= 0).
template <int G>
__device__ __forceinline__ unsigned match_keys(int w, const int (&key)[G]) {
  bool m = false;
#pragma unroll
  for (int k = 0; k < G; ++k) m |= w == key[k];
  return m;
}

// One lane walks its own arc's target row against its vertex's keys in registers: the first eight
// entries and the next four are loaded before any is matched (most of these rows are that short),
// then four at a time with the next four in flight.  -2 marks entries past the row.
template <int G>
__device__ __forceinline__ unsigned lane_walk(const int32_t *__restrict__ row, int d, const int (&key)[G]) {
  unsigned h = 0;
  int w[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) w[r] = r < d ? tc_ld_nc(row + r) : -2;
  int n0 = -2, n1 = -2, n2 = -2, n3 = -2;
  if (d > 8) {
    n0 = tc_ld_nc(row + 8);
    n1 = 9 < d ? tc_ld_nc(row + 9) : -2;
    n2 = 10 < d ? tc_ld_nc(row + 10) : -2;
    n3 = 11 < d ? tc_ld_nc(row + 11) : -2;
  }
#pragma unroll
  for (int r = 0; r < 8; ++r) h += match_keys<G>(w[r], key);
  for (int k = 8; k < d; k += 4) {
    const int m0 = k + 4 < d ? tc_ld_nc(row + k + 4) : -2, m1 = k + 5 < d ? tc_ld_nc(row + k + 5) : -2,
              m2 = k + 6 < d ? tc_ld_nc(row + k + 6) : -2, m3 = k + 7 < d ? tc_ld_nc(row + k + 7) : -2;
    h += match_keys<G>(n0, key) + match_keys<G>(n1, key) + match_keys<G>(n2, key) + match_keys<G>(n3, key);
    n0 = m0; n1 = m1; n2 = m2; n3 = m3;
  }
  return h;
}

// Probe every wedge of a warp whose lanes hold one arc each, lanes [gG, gG+G) belonging to
// vertex g.  Rows of at least 32 * TC_UNROLL entries are walked by the whole warp.  Shorter rows:
// for G <= 8 each lane walks its own row; for G >= 16 the wedges of all groups are flattened into
// one list over the 32 lanes, so a round costs the same whatever the spread of work between
// groups, and a wedge finds its arc by a shuffle binary search and its group's set by the arc's
// lane.
template <int G>
__device__ __forceinline__ void probe_warp_flat(const int32_t *__restrict__ adjC, int s, int dd, int uA,
                                                const int *wtab, unsigned long long &hits,
                                                unsigned long long &wedges) {
  constexpr int U = TC_UNROLL;
  constexpr int LONG = 32 * U;
  const int lane = threadIdx.x & 31;
  wedges += (unsigned)dd;
  unsigned lm = __ballot_sync(TC_FULL_MASK, dd >= LONG);
  while (lm) {
    const int j = __ffs(lm) - 1;
    lm &= lm - 1;
    const int sj = __shfl_sync(TC_FULL_MASK, s, j);
    const int dj = __shfl_sync(TC_FULL_MASK, dd, j);
    const int g = j / G;
    const int32_t *row = adjC + sj;
    int w[U];
#pragma unroll
    for (int r = 0; r < U; ++r) w[r] = lane + r * 32 < dj ? tc_ld_nc(row + lane + r * 32) : -1;
    for (int k = lane; k < dj; k += 32 * U) {
      const int kn = k + 32 * U;
      int wn[U];
#pragma unroll
      for (int r = 0; r < U; ++r) wn[r] = kn + r * 32 < dj ? tc_ld_nc(row + kn + r * 32) : -1;
#pragma unroll
      for (int r = 0; r < U; ++r)
        if (w[r] >= 0) hits += group_has<G>(wtab, g, w[r]);
#pragma unroll
      for (int r = 0; r < U; ++r) w[r] = wn[r];
    }
  }
  // Short rows: flatten.  The nonempty arcs are ranked once (rank c is held by lane c after a
  // gather); a round of 32 consecutive wedges then finds each wedge's arc from the bit mask of
  // arcs starting inside the round: owner rank = arcs started before the round + starts at or
  // before this lane's position - 1.
  const int sd = dd < LONG ? dd : 0;
  if constexpr (G <= 8) {
    // Rows of at most 8 keys: each lane walks its own arc's target row against its vertex's keys
    // held in registers.  A step then costs its longest short row in steps of a few instructions,
    // where flattening costs an owner search per 32 wedges and the ranking of the arcs (Chung-Lu
    // 3.8 M: count 0.408 -> 0.348 ms; 4096x4096 grid: 0.730 -> 0.446 ms; R-MAT 22: 25.1 -> 24.9 ms;
    // keys of 16 in registers were slower on every graph measured).
    int key[G];
#pragma unroll
    for (int k = 0; k < G; ++k) key[k] = __shfl_sync(TC_FULL_MASK, uA, (lane & ~(G - 1)) + k);
    hits += lane_walk<G>(adjC + s, sd, key);
    return;
  }
  const int incl = group_scan_incl<32>(sd, lane);
  const int tot = __shfl_sync(TC_FULL_MASK, incl, 31);
  if (tot == 0) return;
  const unsigned ne = __ballot_sync(TC_FULL_MASK, sd > 0);
  const int nc = __popc(ne);
  const int src = lane < nc ? nth_set_bit(ne, lane) : 0;
  const int src_excl = __shfl_sync(TC_FULL_MASK, incl - sd, src);  // all lanes shuffle, then select
  const int cexcl = lane < nc ? src_excl : 0x7fffffff;
  const int cbase = __shfl_sync(TC_FULL_MASK, s - (incl - sd), src);
  const int cgrp = src / G;
  int before = 0;  // ranked arcs that start before the current round
  const unsigned upto = 0xffffffffu >> (31 - lane);
  for (int k0 = 0; k0 < tot; k0 += 32 * U) {
    int w[U], g[U];
#pragma unroll
    for (int r = 0; r < U; ++r) {
      const int kr = k0 + 32 * r;
      const unsigned starts =
          __reduce_or_sync(TC_FULL_MASK, (cexcl >= kr && cexcl < kr + 32) ? (1u << (cexcl - kr)) : 0u);
      const int c = before + __popc(starts & upto) - 1;
      before += __popc(starts);
      const int cc = c < 0 ? 0 : c;
      const int bj = __shfl_sync(TC_FULL_MASK, cbase, cc);
      g[r] = __shfl_sync(TC_FULL_MASK, cgrp, cc);
      const int k = kr + lane;
      w[r] = k < tot ? tc_ld_nc(adjC + bj + k) : -1;
    }
#pragma unroll
    for (int r = 0; r < U; ++r)
      if (w[r] >= 0) hits += group_has<G>(wtab, g[r], w[r]);
  }
}

// ------------------------------------------------------------------------------------------
// validation / classification
// ------------------------------------------------------------------------------------------
// TC_DEV_BAD_IDS if any of adj[0, m) lies outside [0, bound) (bound < 2^31).  Grid-strided over
// 16-byte loads, two in flight per thread, with scalar loads for the entries before the first
// 16-byte boundary and after the last: a streaming pass limited by bandwidth, not by latency.
__device__ __forceinline__ int ids_out_of_range(const int32_t *__restrict__ adj, int64_t m, int64_t bound,
                                                int64_t tid, int64_t stride) {
  const unsigned ub = (unsigned)bound;
  unsigned any = 0;
  const int64_t lead = (int64_t)(((16u - ((unsigned)(uintptr_t)adj & 15u)) & 15u) >> 2);
  const int64_t head = lead < m ? lead : m;
  if (tid < head) any |= (unsigned)tc_ld_nc(adj + tid) >= ub;
  const int4 *v4 = reinterpret_cast<const int4 *>(adj + head);
  const int64_t n4 = (m - head) >> 2;
  for (int64_t i = tid; i < n4; i += 2 * stride) {
    const int4 a = __ldg(v4 + i);
    const int4 b = i + stride < n4 ? __ldg(v4 + i + stride) : make_int4(0, 0, 0, 0);
    any |= ((unsigned)a.x >= ub) | ((unsigned)a.y >= ub) | ((unsigned)a.z >= ub) | ((unsigned)a.w >= ub) |
           ((unsigned)b.x >= ub) | ((unsigned)b.y >= ub) | ((unsigned)b.z >= ub) | ((unsigned)b.w >= ub);
  }
  for (int64_t i = head + 4 * n4 + tid; i < m; i += stride) any |= (unsigned)tc_ld_nc(adj + i) >= ub;
  return any ? TC_DEV_BAD_IDS : 0;
}

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
  if (check_ids) bad |= ids_out_of_range(adj, m, id_bound, tid, stride);
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  dmax = __reduce_max_sync(TC_FULL_MASK, dmax);
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(&ctl->status, bad);
    atomicMax(&ctl->max_out_degree, dmax);
  }
}

__device__ __forceinline__ int classify(int dA, int dB, int min_deg, int warp_max, int cta_max, int plain) {
  if (dA < min_deg || dB < min_deg) return TC_CLASS_SKIP;
  int d = max(dA, dB);
  if (plain) return d <= warp_max ? TC_CLASS_WARP : d <= cta_max ? TC_CLASS_CTA : TC_CLASS_HUGE;
  if (dA != dB && d > 32) {
    // tables (A) and arc lists (B) differ: the table size picks warp / CTA / spill table, a long
    // arc list alone moves the row to a CTA
    if (dA <= warp_max && dB <= 8 * 32) return TC_CLASS_WARP;
    return dA <= cta_max ? TC_CLASS_CTA : TC_CLASS_HUGE;
  }
  if (d <= 4) return TC_CLASS_G4;
  if (d <= 8) return TC_CLASS_G8;
  if (d <= 16) return TC_CLASS_G16;
  if (d <= 32) return TC_CLASS_G32;
  if (d <= warp_max) return TC_CLASS_WARP;
  if (d <= cta_max) return TC_CLASS_CTA;
  return TC_CLASS_HUGE;
}

// pass 0: histogram of classes.  pass 1: scatter vertex ids into per-class lists.
// Rows outside [row_lo, row_hi) are classed as skipped (their arcs are not counted).
template <int PASS>
__global__ void class_kernel(const int64_t *__restrict__ begA, const int64_t *__restrict__ begB,
                             int64_t rows, int min_deg, int warp_max, int cta_max, int plain,
                             const int *__restrict__ rowmap, const unsigned char *__restrict__ dec,
                             TcControl *ctl, int *__restrict__ lists, ListOffsets off, int64_t row_lo,
                             int64_t row_hi) {
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
      const int64_t va = rowmap ? (int64_t)rowmap[v] : v;
      int dA = (int)(tc_ld_nc(begA + va + 1) - tc_ld_nc(begA + va));
      int dB = (begB == begA && !rowmap) ? dA : (int)(tc_ld_nc(begB + v + 1) - tc_ld_nc(begB + v));
      c = classify(dA, dB, min_deg, warp_max, cta_max, plain);
      if (dec && dA == dB && dA > 32) c = dec[v];  // the learned schedule's decision for long rows
      if (v < row_lo || v >= row_hi) c = TC_CLASS_SKIP;
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

// One CSR (A = B = C, no row map): validation, class histogram and scatter in one kernel.  Class
// c's list is the fixed range [(c-1) rows, c rows) of `lists` (a class holds at most `rows`
// vertices), so no offsets need to reach the host first.  A block owns TC_CC_ROWS consecutive
// rows, TC_CC_PER of them per thread with all their offsets loaded up front: it counts its
// classes in shared memory, reserves its share of every class list with one global atomic per
// class, and scatters from the classes kept in registers.  Rows with bad offsets are flagged and
// left out of every list.  The id check is a separate grid-strided stream over adj.  Rows outside
// [row_lo, row_hi) are validated and measured (maximum out-degree, arcs in long rows) but listed
// in no class: their arcs are not counted.  With alt_lists, every row is also classed under the
// plain split (warp up to TC_PLAIN_WARP_MAX entries, CTA above) and listed there (class c at
// [(c-1) rows, c rows) of alt_lists, sizes in class_count_alt): the host then picks one of the
// two classifications after its one readback, with no second pass.
constexpr int TC_CC_THREADS = 256;
constexpr int TC_CC_PER = 8;
constexpr int TC_CC_ROWS = TC_CC_THREADS * TC_CC_PER;

__global__ void __launch_bounds__(TC_CC_THREADS) check_class_kernel(
    const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t rows, int64_t m, int check_ids,
    int min_deg, int warp_max, int cta_max, int plain, TcControl *ctl, int *__restrict__ lists, int64_t row_lo,
    int64_t row_hi, int *__restrict__ alt_lists) {
  __shared__ int s_hist[TC_NUM_CLASSES];
  __shared__ int s_base[TC_NUM_CLASSES];
  __shared__ int s_hist2[TC_NUM_CLASSES];
  __shared__ int s_base2[TC_NUM_CLASSES];
  const unsigned lt = tc_lanemask_lt();
  const int64_t r0 = (int64_t)blockIdx.x * TC_CC_ROWS;
  int bad = 0, dmax = 0;
  unsigned long long long_arcs = 0;
  if (threadIdx.x < TC_NUM_CLASSES) s_hist[threadIdx.x] = s_hist2[threadIdx.x] = 0;
  long long lo[TC_CC_PER], hi[TC_CC_PER];
#pragma unroll
  for (int k = 0; k < TC_CC_PER; ++k) {
    const int64_t v = r0 + k * TC_CC_THREADS + threadIdx.x;
    lo[k] = v < rows ? tc_ld_nc(beg + v) : 0;
    hi[k] = v < rows ? tc_ld_nc(beg + v + 1) : 0;
  }
  int cls[TC_CC_PER], cls2[TC_CC_PER];
#pragma unroll
  for (int k = 0; k < TC_CC_PER; ++k) {
    cls2[k] = -1;
    const int64_t v = r0 + k * TC_CC_THREADS + threadIdx.x;
    int c = -1;
    if (v < rows) {
      if (hi[k] < lo[k] || lo[k] < 0 || hi[k] > m) {
        bad |= TC_DEV_BAD_OFFSETS;
      } else if (hi[k] - lo[k] >= (1ll << 26)) {
        bad |= TC_DEV_TOO_LARGE;
      } else {
        const int d = (int)(hi[k] - lo[k]);
        dmax = max(dmax, d);
        if (d > TC_LONG_ROW) long_arcs += (unsigned)d;
        c = (v >= row_lo && v < row_hi) ? classify(d, d, min_deg, warp_max, cta_max, plain) : TC_CLASS_SKIP;
        if (alt_lists)
          cls2[k] = (v >= row_lo && v < row_hi) ? classify(d, d, min_deg, TC_PLAIN_WARP_MAX, cta_max, 1) : TC_CLASS_SKIP;
      }
    }
    cls[k] = c;
  }
  __syncthreads();  // s_hist cleared
#pragma unroll
  for (int k = 0; k < TC_CC_PER; ++k) {
    const unsigned peers = __match_any_sync(TC_FULL_MASK, cls[k]);
    if (cls[k] >= 0 && (peers & lt) == 0) atomicAdd(&s_hist[cls[k]], __popc(peers));
    if (alt_lists) {
      const unsigned peers2 = __match_any_sync(TC_FULL_MASK, cls2[k]);
      if (cls2[k] >= 0 && (peers2 & lt) == 0) atomicAdd(&s_hist2[cls2[k]], __popc(peers2));
    }
  }
  __syncthreads();
  if (threadIdx.x < TC_NUM_CLASSES) {
    s_base[threadIdx.x] = s_hist[threadIdx.x] ? atomicAdd(&ctl->class_count[threadIdx.x], s_hist[threadIdx.x]) : 0;
    s_hist[threadIdx.x] = 0;  // from here on: this block's fill cursor per class
    if (alt_lists) {
      s_base2[threadIdx.x] =
          s_hist2[threadIdx.x] ? atomicAdd(&ctl->class_count_alt[threadIdx.x], s_hist2[threadIdx.x]) : 0;
      s_hist2[threadIdx.x] = 0;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < TC_CC_PER; ++k) {
    const int c = cls[k];
    const unsigned peers = __match_any_sync(TC_FULL_MASK, c);
    int at = 0;
    if (c > TC_CLASS_SKIP && (peers & lt) == 0) at = atomicAdd(&s_hist[c], __popc(peers));
    at = __shfl_sync(TC_FULL_MASK, at, __ffs(peers) - 1);
    if (c > TC_CLASS_SKIP)
      lists[(int64_t)(c - 1) * rows + s_base[c] + at + __popc(peers & lt)] = (int)(r0 + k * TC_CC_THREADS + threadIdx.x);
    if (alt_lists) {
      const int c2 = cls2[k];
      const unsigned peers2 = __match_any_sync(TC_FULL_MASK, c2);
      int at2 = 0;
      if (c2 > TC_CLASS_SKIP && (peers2 & lt) == 0) at2 = atomicAdd(&s_hist2[c2], __popc(peers2));
      at2 = __shfl_sync(TC_FULL_MASK, at2, __ffs(peers2) - 1);
      if (c2 > TC_CLASS_SKIP)
        alt_lists[(int64_t)(c2 - 1) * rows + s_base2[c2] + at2 + __popc(peers2 & lt)] =
            (int)(r0 + k * TC_CC_THREADS + threadIdx.x);
    }
  }
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid == 0 && (tc_ld_nc(beg) != 0 || tc_ld_nc(beg + rows) != m)) bad |= TC_DEV_BAD_OFFSETS;
  if (check_ids) bad |= ids_out_of_range(adj, m, rows, tid, (int64_t)gridDim.x * blockDim.x);
  bad = __reduce_or_sync(TC_FULL_MASK, bad);
  dmax = __reduce_max_sync(TC_FULL_MASK, dmax);
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) long_arcs += __shfl_down_sync(TC_FULL_MASK, long_arcs, o);
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(&ctl->status, bad);
    if (dmax) atomicMax(&ctl->max_out_degree, dmax);
    if (long_arcs) atomicAdd(&ctl->long_arcs, long_arcs);
  }
}

// Batch classification: the key of a row is (size class of its graph, degree class), with the
// size class's own thresholds; PASS 0 counts into ctl[s].class_count, PASS 1 scatters at
// ctl[s].class_off (set by batch_offsets_kernel) through ctl[s].class_cursor.
template <int PASS>
__global__ void batch_class_kernel(const int64_t *__restrict__ beg, int64_t rows, const int *__restrict__ graph_of,
                                   const unsigned char *__restrict__ graph_sc, BatchThresholds th, TcControl *ctl,
                                   int *__restrict__ lists) {
  constexpr int K = TC_BATCH_CLASSES * TC_NUM_CLASSES;
  __shared__ int s_hist[K];
  __shared__ int s_base[K];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < rows; base += stride) {
    for (int i = threadIdx.x; i < K; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    const int64_t v = base + threadIdx.x;
    int key = -1;
    if (v < rows) {
      const int d = (int)(tc_ld_nc(beg + v + 1) - tc_ld_nc(beg + v));
      const int sc = graph_sc[graph_of[v]];
      const int c = classify(d, d, 2, th.warp_max[sc], th.cta_max[sc], 0);
      if (c > TC_CLASS_SKIP) key = sc * TC_NUM_CLASSES + c;
    }
    const unsigned peers = __match_any_sync(TC_FULL_MASK, key);
    const int rank = __popc(peers & tc_lanemask_lt());
    int wbase = 0;
    if (key >= 0 && rank == 0) wbase = atomicAdd(&s_hist[key], __popc(peers));
    wbase = __shfl_sync(TC_FULL_MASK, wbase, __ffs(peers) - 1);
    __syncthreads();
    for (int i = threadIdx.x; i < K; i += blockDim.x) {
      if (!s_hist[i]) continue;
      TcControl &cs = ctl[i / TC_NUM_CLASSES];
      if (PASS == 0) atomicAdd(&cs.class_count[i % TC_NUM_CLASSES], s_hist[i]);
      else s_base[i] = atomicAdd(&cs.class_cursor[i % TC_NUM_CLASSES], s_hist[i]);
    }
    __syncthreads();
    if (PASS == 1 && key >= 0)
      lists[ctl[key / TC_NUM_CLASSES].class_off[key % TC_NUM_CLASSES] + s_base[key] + wbase + rank] = (int)v;
    __syncthreads();
  }
}

// List offsets of every (size class, degree class), degree class major: each degree class's rows
// of all size classes are contiguous, so ctl[nsc] (the combined block) describes them as one list
// per degree class, drained by one persistent counting kernel.
__global__ void batch_offsets_kernel(TcControl *ctl, int nsc) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int run = 0;
  for (int c = 0; c < TC_NUM_CLASSES; ++c) {
    ctl[nsc].class_off[c] = run;
    int all = 0;
    for (int s = 0; s < nsc; ++s) {
      ctl[s].class_off[c] = run;
      if (c > TC_CLASS_SKIP) {
        run += ctl[s].class_count[c];
        all += ctl[s].class_count[c];
      }
    }
    ctl[nsc].class_count[c] = all;
  }
}

int launch_batch_classify(int pass, const int64_t *beg, int64_t rows, const int *graph_of,
                          const unsigned char *graph_sc, const BatchThresholds &th, TcControl *ctl, int *lists,
                          int num_sms, cudaStream_t st) {
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((rows + 255) / 256, (int64_t)num_sms * 8));
  if (pass == 0)
    batch_class_kernel<0><<<blocks, 256, 0, st>>>(beg, rows, graph_of, graph_sc, th, ctl, lists);
  else
    batch_class_kernel<1><<<blocks, 256, 0, st>>>(beg, rows, graph_of, graph_sc, th, ctl, lists);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

int launch_batch_offsets(TcControl *ctl, int nsc, cudaStream_t st) {
  batch_offsets_kernel<<<1, 32, 0, st>>>(ctl, nsc);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

// ------------------------------------------------------------------------------------------
// the persistent counting kernel
// ------------------------------------------------------------------------------------------
struct BlockShared {
  unsigned long long count;
  unsigned long long wedges;
  int item;
  int next_batch;
  int n_long;     // deferred long rows of the current CTA vertex
  int next_long;  // claim head over them
  int n_ov;       // quotient table: keys in the overflow list
};

// Neighbour rows at least this long are set aside by the 32-arc batch pass of a CTA vertex and
// then claimed one row per warp, so one batch full of long rows no longer holds up the CTA
// (128 against 256: R-MAT 22 24.98 -> 24.61 ms, R-MAT 26 2270 -> 2262 ms of counting).
constexpr int TC_CTA_LONG = 128;

// Walk one neighbour row with a whole warp: 32 * 2 TC_UNROLL entries per step, next step's loads
// issued before the current step is probed (R-MAT 26: 4 % faster than 4 loads per lane, the bytes
// in flight bounding the walks of rows read from anywhere in the graph).  Steps that lie wholly
// inside the row take no bounds test; the hits of the row are summed in 32 bits (a row has fewer
// than 2^26 entries).
template <class Set>
__device__ __forceinline__ void walk_row_warp(const int32_t *__restrict__ row, int dj, int lane, const Set &set,
                                              unsigned long long &hits) {
  constexpr int U = 2 * TC_UNROLL;  // eight loads in flight per lane: long walks are bound by bytes in flight
  constexpr int STEP = 32 * U;
  unsigned h = 0;
  int k0 = 0;
  if (dj >= STEP) {
    int w[U];
#pragma unroll
    for (int r = 0; r < U; ++r) w[r] = tc_ld_nc(row + lane + r * 32);
    for (; k0 + 2 * STEP <= dj; k0 += STEP) {
      int wn[U];
#pragma unroll
      for (int r = 0; r < U; ++r) wn[r] = tc_ld_nc(row + k0 + STEP + lane + r * 32);
#pragma unroll
      for (int r = 0; r < U; ++r) h += set.has(w[r]);
#pragma unroll
      for (int r = 0; r < U; ++r) w[r] = wn[r];
    }
#pragma unroll
    for (int r = 0; r < U; ++r) h += set.has(w[r]);
    k0 += STEP;
  }
  if (k0 < dj) {  // the last, partial step
    int w[U];
#pragma unroll
    for (int r = 0; r < U; ++r) {
      const int k = k0 + lane + r * 32;
      w[r] = k < dj ? tc_ld_nc(row + k) : -1;
    }
#pragma unroll
    for (int r = 0; r < U; ++r)
      if (w[r] >= 0) h += set.has(w[r]);
  }
  hits += h;
}

__device__ __forceinline__ int ceil_log2_table(int d) {
  // smallest power of two >= 2d, at least 64 slots
  int need = max(2 * d, 64);
  return 32 - __clz(need - 1);
}

// Table row (in A) of work row v.
__device__ __forceinline__ int arow(const CountArgs &p, int v) { return p.rowmap ? p.rowmap[v] : v; }

// Row start and length of v (int: m < 2^31 is enforced on the host).
__device__ __forceinline__ void row_of(const int64_t *__restrict__ beg, int v, int &b, int &d) {
  const long long lo = tc_ld_nc(beg + v), hi = tc_ld_nc(beg + v + 1);
  b = (int)lo;
  d = (int)(hi - lo);
}

// The list of class c (offsets from the host, or computed on the device for batches).
__device__ __forceinline__ const int *class_list(const CountArgs &p, int c) {
  return p.lists + (p.dev_off ? p.ctl->class_off[c] : p.off.off[c]);
}
template <bool BATCH>
__device__ __forceinline__ const int *class_list_t(const CountArgs &p, int c) {
  if constexpr (BATCH) return p.lists + p.ctl->class_off[c];
  else return p.lists + p.off.off[c];
}

// Per-graph attribution of a batch.  Every lane keeps the hits of the graph its warp is
// currently working on; when the warp moves to another graph the warp's sum goes to that graph's
// counter with one atomic.  Calls are warp-uniform (same g in every lane).
struct BatchAcc {
  int cur;
  unsigned long long h;
};

__device__ __forceinline__ void batch_flush(const CountArgs &p, BatchAcc &a) {
  unsigned long long s = a.h;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) s += __shfl_xor_sync(TC_FULL_MASK, s, off);
  if ((threadIdx.x & 31) == 0 && a.cur >= 0 && s) atomicAdd(p.graph_counts + a.cur, s);
  a.h = 0;
}

__device__ __forceinline__ void batch_take(const CountArgs &p, BatchAcc &a, int g, unsigned long long delta) {
  if (g != a.cur) {
    batch_flush(p, a);
    a.cur = g;
  }
  a.h += delta;
}

// One vertex handled by a whole CTA.  `tab` is shared (CTA class) or global (huge class).
// Pass 1: warps claim 32-arc batches from a shared counter; short rows are flattened and probed
// at once, rows of TC_CTA_LONG entries or more are appended to this CTA's long-row list (when
// one is provided and the vertex fits it).  Pass 2: warps claim the long rows one at a time.
// The arcs of a CTA vertex against its table (set): 32-arc batches claimed by the warps, then the
// deferred long rows one per warp.
template <class Set>
__device__ __forceinline__ void cta_arcs(const CountArgs &p, const Set &set, int dA, int bB, int dB, BlockShared &bs,
                                         unsigned long long &hits, unsigned long long &wedges) {
  const int lane = threadIdx.x & 31;
  int2 *longs = (p.long_rows && dB <= p.long_cap) ? p.long_rows + (size_t)blockIdx.x * p.long_cap : nullptr;
  const int nbatch = (dB + 31) >> 5;
  for (;;) {
    int bt = 0;
    if (lane == 0) bt = atomicAdd(&bs.next_batch, 1);
    bt = __shfl_sync(TC_FULL_MASK, bt, 0);
    if (bt >= nbatch) break;
    const int i = (bt << 5) + lane;
    int s = 0, dd = 0;
    if (i < dB) row_of(p.begC, tc_ld_nc(p.adjB + bB + i), s, dd);
    if (p.split && dd > dA) dd = 0;
    if (longs) {
      const bool lg = dd >= TC_CTA_LONG;
      const unsigned lm = __ballot_sync(TC_FULL_MASK, lg);
      if (lm) {
        int at = 0;
        if (lane == 0) at = atomicAdd(&bs.n_long, __popc(lm));
        at = __shfl_sync(TC_FULL_MASK, at, 0);
        if (lg) {
          longs[at + __popc(lm & tc_lanemask_lt())] = make_int2(s, dd);
          wedges += (unsigned)dd;
          dd = 0;
        }
      }
    }
    probe_arcs<32, LongRow<32>::value>(p.adjC, s, dd, lane, set, hits, wedges);
  }
  __syncthreads();
  if (longs) {
    const int n_long = bs.n_long;
    for (;;) {
      int j = 0;
      if (lane == 0) j = atomicAdd(&bs.next_long, 1);
      j = __shfl_sync(TC_FULL_MASK, j, 0);
      if (j >= n_long) break;
      const int2 r = longs[j];
      walk_row_warp(p.adjC + r.x, r.y, lane, set, hits);
    }
    __syncthreads();
  }
}

template <bool SAME>
__device__ void cta_vertex(const CountArgs &p, int v, int *tab, bool smem_table, BlockShared &bs,
                           unsigned long long &hits, unsigned long long &wedges) {
  int bA, dA, bB, dB;
  row_of(p.begA, arow(p, v), bA, dA);
  if (SAME) { bB = bA; dB = dA; } else { row_of(p.begB, v, bB, dB); }
  if (threadIdx.x == 0) {
    bs.next_batch = 0;
    bs.n_long = 0;
    bs.next_long = 0;
  }
  const int bb = smem_table ? q16_log2_buckets(dA, p.key_bits, p.cta_table_bytes) : -1;
  bool ok = true;
  if (bb >= 0) {  // quotient table in shared memory, its overflow list after the buckets
    unsigned *t32 = reinterpret_cast<unsigned *>(tab);
    for (int i = threadIdx.x; i < (4 << bb); i += blockDim.x) t32[i] = 0xFFFFFFFFu;
    if (threadIdx.x == 0) bs.n_ov = 0;
    __syncthreads();
    unsigned short *t16 = reinterpret_cast<unsigned short *>(tab);
    int *ov = tab + (4 << bb);
    for (int i = threadIdx.x; i < dA; i += blockDim.x) {
      const int key = tc_ld_nc(p.adjA + bA + i);
      if (!q16_insert(t16, bb, p.key_bits, key)) {
        const int at = atomicAdd(&bs.n_ov, 1);
        if (at < TC_Q16_OVERFLOW) ov[at] = key;
      }
    }
    __syncthreads();
    const int n_ov = bs.n_ov;
    if (n_ov <= TC_Q16_OVERFLOW) {
      cta_arcs(p, Q16Set{t16, bb, p.key_bits, ov, n_ov}, dA, bB, dB, bs, hits, wedges);
      return;
    }
    // the overflow list ran out: the 32-bit table below (every thread has read n_ov; nothing
    // reads the quotient table any more)
  }
  const int log2 = ceil_log2_table(dA);
  const int T = 1 << log2;
  for (int i = threadIdx.x; i < T; i += blockDim.x) tab[i] = -1;
  __syncthreads();
  for (int i = threadIdx.x; i < dA; i += blockDim.x) ok &= set_insert(tab, log2, tc_ld_nc(p.adjA + bA + i));
  if (!ok) atomicOr(&p.ctl->status, TC_DEV_TABLE_FULL);
  __syncthreads();
  cta_arcs(p, HashSet{tab, log2}, dA, bB, dB, bs, hits, wedges);
}

// One vertex per warp, 32 < out-degree <= warp_max: several 32-arc rounds on a warp table.
template <bool SAME>
__device__ __forceinline__ void warp_vertex(const CountArgs &p, int v, int *warp_tab, unsigned long long &hits,
                                            unsigned long long &wedges) {
  const int lane = threadIdx.x & 31;
  int bA, dA, bB, dB;
  row_of(p.begA, arow(p, v), bA, dA);
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
    if (p.split && dd > dA) dd = 0;
    probe_arcs<32, LongRow<32>::value>(p.adjC, s, dd, lane, set, hits, wedges);
  }
  __syncwarp();
}

// One vertex per G-lane group (G = 4, 8, 16, 32), out-degrees <= G.  The group's row entry uA
// (this lane's element of N+(v), or -1) and the arc's target row (s, dd) were loaded ahead by
// the caller's pipeline.
template <int G, bool SAME>
__device__ __forceinline__ void group_vertex(const CountArgs &p, int uA, int s, int dd, int *wtab,
                                             unsigned long long &hits, unsigned long long &wedges) {
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  const int glane = lane & (G - 1);
  if constexpr (G <= 8) {
    wtab[lane] = uA;  // group g's keys at wtab[gG .. gG+G)
  } else {
    constexpr int LOG2 = (G == 16 ? 4 : 5) + 2;  // 4G slots per group
    int *tab = wtab + g * (4 * G);
#pragma unroll
    for (int i = glane; i < 4 * G; i += G) tab[i] = -1;
    __syncwarp();
    if (uA >= 0) set_insert(tab, LOG2, uA);
  }
  __syncwarp();
  probe_warp_flat<G>(p.adjC, s, dd, uA, wtab, hits, wedges);
  __syncwarp();
}

// Pipeline state of one group for one vertex: the list entry, its row, this lane's row element
// and that element's target row.
struct GroupStage {
  int v, b, d, uA, uB, s, dd;
};

// Drain one group class.  Each warp claims `chunk` steps of 32/G vertices.  Loads run three
// steps ahead: while step t is probed, step t+1's target rows, step t+2's row elements and
// step t+3's row bounds are in flight (the reference walks this chain serially per vertex).
// BATCH: the batch instantiation (per-graph attribution, device list offsets); the single-graph
// kernel carries none of its state.
template <int G, bool SAME, bool REC, bool BATCH>
__device__ void drain_group_class(const CountArgs &p, int c, int *warp_tab, unsigned long long &hits,
                                  unsigned long long &wedges, BatchAcc &acc) {
  constexpr int GPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int g = lane / G;
  const int glane = lane & (G - 1);
  const int n_items = p.ctl->class_count[c];
  const int *list = class_list_t<BATCH>(p, c);
  const int claim = p.chunk * GPW;
  // stage loaders
  auto ld_v = [&](int item, int t1) { return item < t1 ? list[item] : -1; };
  auto ld_row = [&](GroupStage &x) {
    x.b = 0; x.d = 0;
    if (x.v >= 0) row_of(p.begA, SAME ? x.v : arow(p, x.v), x.b, x.d);
  };
  auto ld_elem = [&](GroupStage &x) {
    x.uA = glane < x.d ? tc_ld_nc(p.adjA + x.b + glane) : -1;
    if (SAME) {
      x.uB = x.uA;
    } else {
      int bB = 0, dB = 0;
      if (x.v >= 0) row_of(p.begB, x.v, bB, dB);
      x.uB = glane < dB ? tc_ld_nc(p.adjB + bB + glane) : -1;
    }
  };
  auto ld_target = [&](GroupStage &x) {
    x.s = 0; x.dd = 0;
    if (x.uB >= 0) row_of(p.begC, x.uB, x.s, x.dd);
    if (p.split && x.dd > x.d) x.dd = 0;  // counted from u's side in the second pass
  };
  for (;;) {
    int t0 = 0;
    if (lane == 0) t0 = atomicAdd(&p.ctl->class_next[c], claim);
    t0 = __shfl_sync(TC_FULL_MASK, t0, 0);
    if (t0 >= n_items) break;
    const int t1 = min(t0 + claim, n_items);
    GroupStage s0, s1, s2;
    s0.v = ld_v(t0 + g, t1);
    s1.v = ld_v(t0 + GPW + g, t1);
    s2.v = ld_v(t0 + 2 * GPW + g, t1);
    ld_row(s0);
    ld_row(s1);
    ld_elem(s0);
    ld_target(s0);
    ld_elem(s1);
    ld_row(s2);
    for (int t = t0; t < t1; t += GPW) {
      GroupStage s3;
      s3.v = ld_v(t + 3 * GPW + g, t1);
      ld_target(s1);  // row elements of t+1 arrived during the previous step
      ld_elem(s2);
      ld_row(s3);
      const long long t_start = REC ? clock64() : 0;
      if constexpr (!BATCH) {
        group_vertex<G, SAME>(p, s0.uA, s0.s, s0.dd, warp_tab, hits, wedges);
      } else {
        // a batch: one pass per graph present in this step (almost always one), the other
        // groups' vertices masked out, so every hit of a pass belongs to that pass's graph
        const int gid = s0.v >= 0 ? p.graph_of[s0.v] : -1;
        unsigned pending = __ballot_sync(TC_FULL_MASK, gid >= 0);
        while (pending) {
          const int gx = __shfl_sync(TC_FULL_MASK, gid, __ffs(pending) - 1);
          const bool mine = gid == gx;
          const unsigned long long h0 = hits;
          group_vertex<G, SAME>(p, mine ? s0.uA : -1, s0.s, mine ? s0.dd : 0, warp_tab, hits, wedges);
          batch_take(p, acc, gx, hits - h0);
          pending &= ~__ballot_sync(TC_FULL_MASK, mine);
        }
      }
      if (REC) {
        // the step's cycles, shared among its vertices in proportion to their wedges
        const long long dt = clock64() - t_start;
        int wv = s0.dd;
#pragma unroll
        for (int off = G / 2; off >= 1; off >>= 1) wv += __shfl_xor_sync(TC_FULL_MASK, wv, off, G);
        int wstep = s0.dd;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) wstep += __shfl_xor_sync(TC_FULL_MASK, wstep, off);
        if (glane == 0 && s0.v >= 0)
          p.cycles[s0.v] = (unsigned long long)(wstep > 0 ? (double)dt * wv / wstep : (double)dt / GPW);
      }
      s0 = s1;
      s1 = s2;
      s2 = s3;
    }
  }
}

// Two register budgets: up to 1024 threads per CTA (reference launch shape), or <= 256 threads
// with at least TC_MIN_CTAS_256 CTAs resident per SM (the default shape).
constexpr int TC_MIN_CTAS_256 = 5;

template <bool SAME, bool REC, int MAXT, int MINB, bool BATCH>
__global__ void __launch_bounds__(MAXT, MINB) count_kernel(CountArgs p) {
  extern __shared__ int smem[];
  __shared__ BlockShared bs;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) bs.count = bs.wedges = 0;
  unsigned long long hits = 0, wedges = 0;
  BatchAcc acc{-1, 0};

  // Phase A: CTA-granularity vertices, largest class first.
  for (int c = TC_CLASS_HUGE; c >= TC_CLASS_CTA; --c) {
    const int n_items = p.ctl->class_count[c];
    if (n_items == 0) continue;
    if (c == TC_CLASS_HUGE && (int)blockIdx.x >= p.huge_blocks) continue;
    const int *list = class_list_t<BATCH>(p, c);
    int *tab = (c == TC_CLASS_HUGE) ? p.huge_tables + (size_t)blockIdx.x * ((size_t)1 << p.huge_log2)
                                    : smem;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) bs.item = atomicAdd(&p.ctl->class_next[c], 1);
      __syncthreads();
      const int t = bs.item;
      if (t >= n_items) break;
      const int v = list[t];
      if (c == TC_CLASS_HUGE && p.hub_max_degree > 0) {  // counted by hub_kernel instead
        int hb, hd;
        row_of(p.begA, arow(p, v), hb, hd);
        if (hd <= p.hub_max_degree) continue;
      }
      const long long t_start = REC ? clock64() : 0;
      const unsigned long long h0 = hits;
      cta_vertex<SAME>(p, v, tab, c == TC_CLASS_CTA, bs, hits, wedges);
      if (REC && threadIdx.x == 0) p.cycles[v] = (unsigned long long)(clock64() - t_start);
      if constexpr (BATCH) batch_take(p, acc, p.graph_of[v], hits - h0);
    }
  }
  __syncthreads();

  // Phase B: warp and sub-warp granularity.
  int *warp_tab = smem + warp * p.warp_slots;
  {
    const int c = TC_CLASS_WARP;
    const int n_items = p.ctl->class_count[c];
    const int *list = class_list_t<BATCH>(p, c);
    for (;;) {
      int t0 = 0;
      // warp-class vertices are large: claim them one at a time unless the chunk is very coarse
      const int claim = max(1, p.chunk / 8);
      if (lane == 0) t0 = atomicAdd(&p.ctl->class_next[c], claim);
      t0 = __shfl_sync(TC_FULL_MASK, t0, 0);
      if (t0 >= n_items) break;
      const int t1 = min(t0 + claim, n_items);
      for (int t = t0; t < t1; ++t) {
        const int v = list[t];
        const long long t_start = REC ? clock64() : 0;
        const unsigned long long h0 = hits;
        warp_vertex<SAME>(p, v, warp_tab, hits, wedges);
        if (REC && lane == 0) p.cycles[v] = (unsigned long long)(clock64() - t_start);
        if constexpr (BATCH) batch_take(p, acc, p.graph_of[v], hits - h0);
      }
    }
  }
  drain_group_class<32, SAME, REC, BATCH>(p, TC_CLASS_G32, warp_tab, hits, wedges, acc);
  drain_group_class<16, SAME, REC, BATCH>(p, TC_CLASS_G16, warp_tab, hits, wedges, acc);
  drain_group_class<8, SAME, REC, BATCH>(p, TC_CLASS_G8, warp_tab, hits, wedges, acc);
  drain_group_class<4, SAME, REC, BATCH>(p, TC_CLASS_G4, warp_tab, hits, wedges, acc);
  if constexpr (BATCH) batch_flush(p, acc);

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
// hub rows in shared memory: one CTA, or a thread-block cluster (distributed shared memory)
// ------------------------------------------------------------------------------------------
// A hub row's table (2^log2 slots, as for a CTA table) is split evenly over the C CTAs of a
// cluster: slot s lives in CTA s >> share_log2 at index s & (2^share_log2 - 1).  Inserts and
// probes reach the other CTAs' slots through distributed shared memory; the cluster's warps claim
// the hub's 32-arc batches from a counter in CTA 0's shared memory.  C = 1 is a single CTA with a
// table larger than the persistent kernel's.
namespace cg = cooperative_groups;

struct DsmemSet {
  int *local;
  int log2;        // table slots: 2^log2
  int share_log2;  // slots per CTA
  __device__ __forceinline__ int *slot(unsigned s) const {
    return cg::this_cluster().map_shared_rank(local, (int)(s >> share_log2)) + (s & ((1u << share_log2) - 1u));
  }
  __device__ __forceinline__ int has(int key) const {
    const unsigned bmask = (1u << (log2 - 2)) - 1u;
    unsigned b = tc_hash((unsigned)key, log2 - 2);
    for (unsigned it = 0; it <= bmask; ++it) {
      const int4 q = *reinterpret_cast<const int4 *>(slot(b << 2));
      if (q.x == key || q.y == key || q.z == key || q.w == key) return 1;
      if ((q.x | q.y | q.z | q.w) < 0) return 0;
      b = (b + 1u) & bmask;
    }
    return 0;
  }
  __device__ __forceinline__ bool insert(int key) const {
    const unsigned mask = (1u << log2) - 1u;
    unsigned h = tc_hash((unsigned)key, log2 - 2) << 2;
    for (unsigned it = 0; it <= mask; ++it) {
      const int prev = atomicCAS(slot(h), -1, key);
      if (prev == -1 || prev == key) return true;
      h = (h + 1u) & mask;
    }
    return false;
  }
};

// ---- TMA bulk copy (cp.async.bulk) into shared memory, completion on an mbarrier ----
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: arm the barrier for `bytes` of transfers (the phase completes once they arrive).
__device__ __forceinline__ void mbar_arm(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One thread: arm the barrier for `bytes` and start the copy of [src, src + bytes) to dst.
// src and dst 16-byte aligned, bytes a multiple of 16 (< 2^20).
// The fence orders this CTA's earlier generic-proxy reads of dst before the copy's writes.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_arm(bar, bytes);
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Bounds of the copy waits, in clock64 cycles: about a second at the GB300 clock, and a few
// thousand for the failure-detection test (whose barrier nothing completes).
constexpr long long TC_WAIT_CYCLES = 2ll << 30;
constexpr long long TC_TEST_WAIT_CYCLES = 4096;

// Wait for the barrier's phase `parity` to complete, giving up after `limit` clock64 cycles
// (returns false then; the caller records TC_DEV_WAIT_LIMIT and stops using the copies).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, long long limit) {
  const long long t0 = clock64();
  for (;;) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// Persistent over the huge list: a cluster claims hubs one at a time from a counter (rank 0 claims,
// the cluster reads the claim from its shared memory), so the heaviest-first order of the list
// becomes a longest-first schedule instead of a fixed round-robin whose heaviest clusters set the
// tail; rows longer than p.hub_max_degree are left to the main kernel's spill tables.  Every
// cluster.sync() is reached by all CTAs of the cluster (the claim, the loop exit and the skip
// test are the same for all of them); no remote access happens before the first sync of a hub,
// and none after the final sync.
// Each CTA stages its contiguous share of the hub row with one TMA bulk copy (the 16-byte aligned
// interior; the ragged ends, at most 3 entries each, by plain loads) and inserts from shared
// memory.  Dynamic shared memory: the table share (2^share_log2_max ints) then the staging buffer.
// A copy whose bounded wait runs out may still be in flight into the staging buffer: the CTA
// reports TC_DEV_WAIT_LIMIT, reads that share with plain loads, never touches the staging buffer
// again, and before it exits waits once more (bounded) for the abandoned copy, so its shared
// memory is not released under a write still landing.  With p.test_wait_expiry the barrier is
// armed without a copy, so the wait runs out with nothing in flight.
template <bool SAME>
__global__ void __launch_bounds__(512, 2) hub_kernel(CountArgs p, int log2C, int share_log2_max) {
  extern __shared__ __align__(16) int smem[];
  __shared__ int next_batch;
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int tma_ok;
  __shared__ int abandoned;  // 1 + parity of a barrier phase whose copy this CTA stopped waiting for
  __shared__ int n_ov;       // quotient table: keys in the overflow list
  __shared__ int claimed;    // rank 0: the hub this cluster claimed
  // dynamic shared memory: the table share, the quotient table's overflow list, the staging buffer
  int *ov = smem + (1 << share_log2_max);
  int *stage = ov + TC_Q16_OVERFLOW;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    tma_ok = ((reinterpret_cast<uintptr_t>(p.adjA) & 15) == 0);  // 16-byte aligned base: copy the interior
    abandoned = 0;
  }
  __syncthreads();
  unsigned parity = 0;
  cg::cluster_group cl = cg::this_cluster();
  const int C = 1 << log2C;
  const int rank = (int)cl.block_rank();
  const int lane = threadIdx.x & 31;
  const int n_items = p.ctl->class_count[TC_CLASS_HUGE];
  const int *list = class_list(p, TC_CLASS_HUGE);
  int *ctr = cl.map_shared_rank(&next_batch, 0);
  unsigned long long hits = 0, wedges = 0;
  // hub claims: class_next[TC_CLASS_SKIP], a head no counting queue uses
  int *claim_src = cl.map_shared_rank(&claimed, 0);
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) claimed = atomicAdd(&p.ctl->class_next[TC_CLASS_SKIP], 1);
    cl.sync();
    const int t = *claim_src;
    cl.sync();  // every CTA has read the claim before rank 0 makes the next one
    if (t >= n_items) break;
    const int v = list[t];
    int bA, dA, bB, dB;
    row_of(p.begA, arow(p, v), bA, dA);
    if (dA > p.hub_max_degree) continue;  // the same in every CTA of the cluster
    if (SAME) { bB = bA; dB = dA; } else { row_of(p.begB, v, bB, dB); }
    const long long t_start = p.cycles ? clock64() : 0;
    const int log2 = ceil_log2_table(dA);
    const DsmemSet set{smem, log2, log2 - log2C};
    const int share = 1 << (log2 - log2C);
    // one CTA: a quotient table (see Q16Set) when the ids allow it, else the 32-bit table
    const int bb = log2C == 0 ? q16_log2_buckets(dA, p.key_bits, (4 << share_log2_max) + 4 * TC_Q16_OVERFLOW) : -1;
    unsigned short *t16 = reinterpret_cast<unsigned short *>(smem);
    if (bb >= 0) {
      for (int i = threadIdx.x; i < (4 << bb); i += blockDim.x) smem[i] = -1;
    } else {
      for (int i = threadIdx.x; i < share; i += blockDim.x) smem[i] = -1;
    }
    if (threadIdx.x == 0) n_ov = 0;
    if (rank == 0 && threadIdx.x == 0) next_batch = 0;
    cl.sync();
    bool ok = true;
    auto insert = [&](int key) -> bool {
      if (bb < 0) return set.insert(key);
      if (!q16_insert(t16, bb, p.key_bits, key)) {
        const int at = atomicAdd(&n_ov, 1);
        if (at < TC_Q16_OVERFLOW) ov[at] = key;
      }
      return true;
    };
    {  // this CTA's share of the row: entries [lo, hi)
      const int per = (dA + C - 1) >> log2C;
      const int lo = min(rank * per, dA), hi = min(lo + per, dA);
      const long long a0 = (long long)bA + lo, a1 = (long long)bA + hi;
      const long long i0 = (a0 + 3) & ~3ll, i1 = a1 & ~3ll;  // aligned interior [i0, i1)
      if (tma_ok && i1 > i0) {
        const bool copy = !p.test_wait_expiry;
        if (threadIdx.x == 0) {
          if (copy) bulk_copy_g2s(stage, p.adjA + i0, (unsigned)(i1 - i0) * 4u, &bar);
          else mbar_arm(&bar, (unsigned)(i1 - i0) * 4u);  // nothing will arrive
        }
        for (long long i = a0 + threadIdx.x; i < i0; i += blockDim.x) ok &= insert(tc_ld_nc(p.adjA + i));
        for (long long i = i1 + threadIdx.x; i < a1; i += blockDim.x) ok &= insert(tc_ld_nc(p.adjA + i));
        const bool arrived = mbar_wait(&bar, parity, copy ? TC_WAIT_CYCLES : TC_TEST_WAIT_CYCLES);
        parity ^= 1u;
        if (arrived) {
          for (int i = threadIdx.x; i < (int)(i1 - i0); i += blockDim.x) ok &= insert(stage[i]);
        } else {  // give up on the copy: report it and read the interior directly
          if (threadIdx.x == 0) atomicOr(&p.ctl->status, TC_DEV_WAIT_LIMIT);
          for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) ok &= insert(tc_ld_nc(p.adjA + i));
        }
        __syncthreads();  // the staging buffer is free again, and every thread saw the same outcome
        if (threadIdx.x == 0 && !arrived) {
          tma_ok = 0;  // no more copies (every thread sees it after the barrier below)
          if (copy) abandoned = 1 + (int)(parity ^ 1u);
        }
        __syncthreads();
      } else {
        for (long long i = a0 + threadIdx.x; i < a1; i += blockDim.x) ok &= insert(tc_ld_nc(p.adjA + i));
      }
    }
    if (!ok) atomicOr(&p.ctl->status, TC_DEV_TABLE_FULL);
    cl.sync();
    bool use16 = bb >= 0;
    if (use16 && n_ov > TC_Q16_OVERFLOW) {  // the overflow list ran out (one CTA): a 32-bit table
      use16 = false;
      __syncthreads();
      for (int i = threadIdx.x; i < share; i += blockDim.x) smem[i] = -1;
      __syncthreads();
      for (int i = threadIdx.x; i < dA; i += blockDim.x) ok &= set.insert(tc_ld_nc(p.adjA + bA + i));
      if (!ok) atomicOr(&p.ctl->status, TC_DEV_TABLE_FULL);
      __syncthreads();
    }
    auto probe_all = [&](const auto &tset) {
      const int nbatch = (dB + 31) >> 5;
      for (;;) {
        int bt = 0;
        if (lane == 0) bt = atomicAdd(ctr, 1);
        bt = __shfl_sync(TC_FULL_MASK, bt, 0);
        if (bt >= nbatch) break;
        const int i = (bt << 5) + lane;
        int s = 0, dd = 0;
        if (i < dB) row_of(p.begC, tc_ld_nc(p.adjB + bB + i), s, dd);
        if (p.split && dd > dA) dd = 0;
        probe_arcs<32, LongRow<32>::value>(p.adjC, s, dd, lane, tset, hits, wedges);
      }
    };
    if (use16) probe_all(Q16Set{t16, bb, p.key_bits, ov, n_ov});
    else probe_all(set);
    cl.sync();  // every probe of this hub is done before any share is cleared again
    if (p.cycles && rank == 0 && threadIdx.x == 0) p.cycles[v] = (unsigned long long)(clock64() - t_start);
  }
  if (abandoned && threadIdx.x == 0 && !mbar_wait(&bar, (unsigned)(abandoned - 1), TC_WAIT_CYCLES))
    atomicOr(&p.ctl->status, TC_DEV_WAIT_LIMIT);  // already set when it was abandoned; nothing else to do
  cl.sync();  // no CTA leaves while another may still read its shared memory
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    hits += __shfl_down_sync(TC_FULL_MASK, hits, off);
    wedges += __shfl_down_sync(TC_FULL_MASK, wedges, off);
  }
  if (lane == 0 && hits) atomicAdd(&p.ctl->count, hits);
  if (lane == 0 && wedges) atomicAdd(&p.ctl->wedges, wedges);
}

// Kernel attributes live per device and function, and every set is a driver call (several per
// counting call otherwise, on the host path between classification and the count launch).  Each
// (device, function, attribute) remembers what it was last set to; the dynamic shared memory
// limit only ever grows.  Occupancy results are memoised per (device, kernel, threads, bytes).
// Every attribute of the count kernels is set through here.
struct AttrCache {
  std::mutex mu;
  std::map<std::tuple<int, const void *, int>, int> val;
  std::map<std::tuple<int, const void *, int, size_t>, int> occ;
};
static AttrCache &attr_cache() {
  static AttrCache c;
  return c;
}

static cudaError_t set_attr(const void *fn, cudaFuncAttribute a, int v, bool grow_only = false) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  AttrCache &c = attr_cache();
  std::lock_guard<std::mutex> lk(c.mu);
  const auto key = std::make_tuple(dev, fn, (int)a);
  auto it = c.val.find(key);
  if (it != c.val.end() && (it->second == v || (grow_only && it->second > v))) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, a, v);
  if (e == cudaSuccess) c.val[key] = v;
  else c.val.erase(key);
  return e;
}

int launch_hub(bool same, const CountArgs &a, int max_log2, int log2C, int clusters, cudaStream_t st) {
  // table share + staging for one CTA's share of the longest row (plus alignment slack)
  const int share_log2 = max_log2 - log2C;
  const size_t stage_ints = (((size_t)a.hub_max_degree + (1u << log2C) - 1) >> log2C) + 8;
  const size_t smem = ((size_t)4 << share_log2) + 4 * (size_t)TC_Q16_OVERFLOW + 4 * stage_ints;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters << log2C));
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1u << log2C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if (same) {
    e = set_attr((const void *)hub_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem, true);
    if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, hub_kernel<true>, a, log2C, share_log2);
  } else {
    e = set_attr((const void *)hub_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem, true);
    if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, hub_kernel<false>, a, log2C, share_log2);
  }
  TC_CUDA_TRY(e);
  TC_NOTE_LAUNCH();
  return TRUST_TC_OK;
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
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

int launch_check_classify(const int64_t *beg, const int32_t *adj, int64_t rows, int64_t m, int check_ids,
                          int min_deg, int warp_max, int cta_max, int schedule, TcControl *ctl, int *lists,
                          int num_sms, cudaStream_t st, int64_t row_lo, int64_t row_hi, int *alt_lists) {
  // one block per TC_CC_ROWS rows; blocks past the last row only check ids (few rows, many arcs)
  int64_t blocks = std::max<int64_t>(1, (rows + TC_CC_ROWS - 1) / TC_CC_ROWS);
  if (check_ids) blocks = std::max<int64_t>(blocks, std::min<int64_t>((m + 4095) / 4096, (int64_t)num_sms * 8));
  if (blocks > 0x7fffffff) return TRUST_TC_E_TOO_LARGE;
  check_class_kernel<<<(unsigned)blocks, TC_CC_THREADS, 0, st>>>(beg, adj, rows, m, check_ids, min_deg, warp_max,
                                                                 cta_max, schedule == TRUST_TC_SCHED_PLAIN, ctl, lists,
                                                                 row_lo, row_hi < 0 ? rows : row_hi, alt_lists);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

int launch_classify(int pass, const int64_t *begA, const int64_t *begB, int64_t rows, int min_deg,
                    int warp_max, int cta_max, TcControl *ctl, int *lists, const ListOffsets &off,
                    int num_sms, cudaStream_t st, int schedule, const int *rowmap, const unsigned char *dec,
                    int64_t row_lo, int64_t row_hi) {
  int blocks = (int)std::min<int64_t>((rows + 255) / 256, (int64_t)num_sms * 8);
  blocks = std::max(blocks, 1);
  const int plain = schedule == TRUST_TC_SCHED_PLAIN;
  if (row_hi < 0) row_hi = rows;
  if (pass == 0)
    class_kernel<0><<<blocks, 256, 0, st>>>(begA, begB, rows, min_deg, warp_max, cta_max, plain, rowmap, dec, ctl,
                                            lists, off, row_lo, row_hi);
  else
    class_kernel<1><<<blocks, 256, 0, st>>>(begA, begB, rows, min_deg, warp_max, cta_max, plain, rowmap, dec, ctl,
                                            lists, off, row_lo, row_hi);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

// The occupancy query honours the kernel's preferred carveout, which a previous call may have
// set low (a graph needing little shared memory); it runs with the carveout at the maximum, or
// the query (and so the grid) would be limited by the last graph's carveout.
template <bool SAME, int MAXT, int MINB>
static cudaError_t occupancy_of(int threads, size_t smem_bytes, int *blocks_per_sm) {
  cudaError_t e = cudaSuccess;
  const void *fns[3] = {(const void *)count_kernel<SAME, false, MAXT, MINB, false>,
                        (const void *)count_kernel<SAME, true, MAXT, MINB, false>,
                        (const void *)count_kernel<SAME, false, MAXT, MINB, SAME>};
  for (const void *fn : fns)
    if (e == cudaSuccess) e = set_attr(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes, true);
  if (e != cudaSuccess) return e;
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  const auto key = std::make_tuple(dev, fns[0], threads, smem_bytes);
  {
    AttrCache &c = attr_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.occ.find(key);
    if (it != c.occ.end()) {
      *blocks_per_sm = it->second;
      return cudaSuccess;
    }
  }
  for (const void *fn : fns)
    if (e == cudaSuccess) e = set_attr(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, count_kernel<SAME, false, MAXT, MINB, false>, threads,
                                                      smem_bytes);
  if (e == cudaSuccess) {
    AttrCache &c = attr_cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.occ[key] = *blocks_per_sm;
  }
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

template <bool SAME, int MAXT, int MINB>
static cudaError_t carveout_of(int pct) {
  cudaError_t e = cudaSuccess;
  for (const void *fn : {(const void *)count_kernel<SAME, false, MAXT, MINB, false>,
                         (const void *)count_kernel<SAME, true, MAXT, MINB, false>,
                         (const void *)count_kernel<SAME, false, MAXT, MINB, SAME>})
    if (e == cudaSuccess) e = set_attr(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
  return e;
}

int set_count_kernel_carveout(bool same, int threads, size_t smem_bytes, int per_sm) {
  // per-CTA reservation of 1 KiB on top of the dynamic and static shared memory
  const double need = (double)per_sm * (double)(smem_bytes + 2048);
  int pct = (int)(100.0 * need / (228.0 * 1024.0)) + 1;
  pct = std::min(std::max(pct, 0), 100);
  cudaError_t e;
  if (threads <= 256)
    e = same ? carveout_of<true, 256, TC_MIN_CTAS_256>(pct) : carveout_of<false, 256, TC_MIN_CTAS_256>(pct);
  else
    e = same ? carveout_of<true, 1024, 1>(pct) : carveout_of<false, 1024, 1>(pct);
  TC_CUDA_TRY(e);
  return TRUST_TC_OK;
}

template <bool SAME, int MAXT, int MINB>
static void launch_one(const CountArgs &a, int blocks, int threads, size_t smem_bytes, cudaStream_t st) {
  if (SAME && a.graph_of)  // batches: one graph CSR, no cycle recording
    count_kernel<SAME, false, MAXT, MINB, SAME><<<blocks, threads, smem_bytes, st>>>(a);
  else if (a.cycles)
    count_kernel<SAME, true, MAXT, MINB, false><<<blocks, threads, smem_bytes, st>>>(a);
  else
    count_kernel<SAME, false, MAXT, MINB, false><<<blocks, threads, smem_bytes, st>>>(a);
  TC_NOTE_LAUNCH();
}

int launch_count(bool same, const CountArgs &a, int blocks, int threads, size_t smem_bytes,
                 cudaStream_t st) {
  if (threads <= 256) {
    if (same) launch_one<true, 256, TC_MIN_CTAS_256>(a, blocks, threads, smem_bytes, st);
    else launch_one<false, 256, TC_MIN_CTAS_256>(a, blocks, threads, smem_bytes, st);
  } else {
    if (same) launch_one<true, 1024, 1>(a, blocks, threads, smem_bytes, st);
    else launch_one<false, 1024, 1>(a, blocks, threads, smem_bytes, st);
  }
  TC_CUDA_TRY(cudaGetLastError());
  return TRUST_TC_OK;
}

}  // namespace tc

// tc_prep.cu — GPU preprocessing: edge pairs -> oriented, renumbered CSR.
//
// Moves the reference's CPU preprocessing onto the GPU:
//   Preprocess/fromDirectToUndirect.cpp:53-109  compact ids, (min,max) pairs, dedupe
//   Preprocess/preprocess_outdegree.cpp:79-98   orient each edge from lower to higher degree
//   Preprocess/preprocess_outdegree.cpp:186-222 renumber (out-degree descending) and write CSR
// with two deliberate changes: ties are broken by vertex id (the reference's std::sort leaves
// them unspecified) and each row is sorted ascending (the reference writes rows unsorted, :213).
// Vertices without edges are dropped (the reference keeps a self-loop-only vertex as an isolated
// row).  Every step is a stable LSD radix sort, a scan, or an elementwise kernel.
#include <algorithm>
#include <vector>

#include "tc_internal.h"

namespace tc {

typedef unsigned long long u64;
typedef unsigned int u32;

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // keys per CTA per pass

// ------------------------------------------------------------------------------------------
// scans (exclusive, tile of 4096 per CTA, reduce-then-scan)
// ------------------------------------------------------------------------------------------
template <typename T>
__device__ T block_excl_scan(T x, T *total) {
  __shared__ T warp_tot[RS_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T incl = x;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    T y = __shfl_up_sync(TC_FULL_MASK, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    T w = lane < RS_THREADS / 32 ? warp_tot[lane] : T(0);
    T wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      T y = __shfl_up_sync(TC_FULL_MASK, wi, off);
      if (lane >= off) wi += y;
    }
    if (lane < RS_THREADS / 32) warp_tot[lane] = wi - w;
    if (lane == RS_THREADS / 32 - 1) *total = wi;
  }
  __syncthreads();
  T r = warp_tot[warp] + incl - x;
  __syncthreads();
  return r;
}

template <typename T>
__global__ void scan_reduce_kernel(const T *__restrict__ in, int64_t n, T *__restrict__ sums) {
  __shared__ T tot;
  const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)threadIdx.x * RS_ITEMS;
  T s = 0;
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j)
    if (base + j < n) s += in[base + j];
  block_excl_scan<T>(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void scan_down_kernel(const T *in, T *out, int64_t n, const T *__restrict__ offs) {
  __shared__ T tot;
  const int64_t base = (int64_t)blockIdx.x * RS_TILE + (int64_t)threadIdx.x * RS_ITEMS;
  T v[RS_ITEMS];
  T s = 0;
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    v[j] = base + j < n ? in[base + j] : T(0);
    s += v[j];
  }
  T run = block_excl_scan<T>(s, &tot) + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
}

// Exclusive scan of n elements (in may equal out).  Returns the total through *total_out
// (device-to-host read, synchronising `st`) when total_out is not null.
template <typename T>
static int scan_exclusive(const T *in, T *out, int64_t n, cudaStream_t st, T *total_out) {
  if (n <= 0) {
    if (total_out) *total_out = 0;
    return TRUST_TC_OK;
  }
  T last_in = 0;
  if (total_out) TC_CUDA_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(T), cudaMemcpyDeviceToHost, st));
  if (total_out) TC_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t nb = (n + RS_TILE - 1) / RS_TILE;
  T *sums = nullptr;
  if (nb > 1) {
    TC_CUDA_TRY(cudaMallocAsync((void **)&sums, sizeof(T) * nb, st));
    scan_reduce_kernel<T><<<(unsigned)nb, RS_THREADS, 0, st>>>(in, n, sums);
    TC_NOTE_LAUNCH();
    TC_CUDA_TRY(cudaGetLastError());
    int rc = scan_exclusive<T>(sums, sums, nb, st, (T *)nullptr);
    if (rc) return rc;
  }
  scan_down_kernel<T><<<(unsigned)nb, RS_THREADS, 0, st>>>(in, out, n, sums);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaGetLastError());
  if (sums) TC_CUDA_TRY(cudaFreeAsync(sums, st));
  if (total_out) {
    T last_out = 0;
    TC_CUDA_TRY(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(T), cudaMemcpyDeviceToHost, st));
    TC_CUDA_TRY(cudaStreamSynchronize(st));
    *total_out = last_out + last_in;
  }
  return TRUST_TC_OK;
}

int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t st, int64_t *total) {
  return scan_exclusive<int64_t>(in, out, n, st, total);
}

// ------------------------------------------------------------------------------------------
// stable LSD radix sort of u64 keys, 8-bit digits
// ------------------------------------------------------------------------------------------
__global__ void rs_hist_kernel(const u64 *__restrict__ keys, int64_t n, int shift, u32 *__restrict__ counts,
                               u32 nblocks) {
  __shared__ u32 h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int r = 0; r < RS_ITEMS; ++r) {
    int64_t i = base + r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void rs_scatter_kernel(const u64 *__restrict__ in, u64 *__restrict__ out, int64_t n, int shift,
                                  const u32 *__restrict__ offs, u32 nblocks) {
  constexpr int NW = RS_THREADS / 32;
  __shared__ u32 cnt[NW][256];
  __shared__ u32 pre[NW][256];
  __shared__ u32 run[256];
  __shared__ u32 gbase[256];
  const int tid = threadIdx.x, warp = tid >> 5;
  run[tid] = 0;
  gbase[tid] = offs[(size_t)tid * nblocks + blockIdx.x];
#pragma unroll
  for (int w = 0; w < NW; ++w) cnt[w][tid] = 0;
  __syncthreads();
  const unsigned lt = tc_lanemask_lt();
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  for (int r = 0; r < RS_ITEMS; ++r) {
    const int64_t i = base + r * RS_THREADS + tid;
    const bool valid = i < n;
    const u64 key = valid ? in[i] : 0ull;
    const int d = valid ? (int)((key >> shift) & 255u) : 256;
    const unsigned peers = __match_any_sync(TC_FULL_MASK, d);
    const u32 lrank = __popc(peers & lt);
    if (valid && lrank == 0) cnt[warp][d] = __popc(peers);
    __syncthreads();
    u32 s = run[tid];
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      u32 c = cnt[w][tid];
      pre[w][tid] = s;
      s += c;
      cnt[w][tid] = 0;
    }
    run[tid] = s;
    __syncthreads();
    if (valid) out[gbase[d] + pre[warp][d] + lrank] = key;
  }
}

// Sort `keys` (n < 2^32) by the 8-bit digits starting at each listed bit shift (low first).
// `tmp` has room for n keys.  The result ends in `keys`.
static int radix_sort(u64 *keys, u64 *tmp, int64_t n, const std::vector<int> &shifts, cudaStream_t st) {
  if (n <= 1 || shifts.empty()) return TRUST_TC_OK;
  if (n >= ((int64_t)1 << 32)) return TRUST_TC_E_TOO_LARGE;
  const u32 nb = (u32)((n + RS_TILE - 1) / RS_TILE);
  u32 *counts = nullptr;
  TC_CUDA_TRY(cudaMallocAsync((void **)&counts, sizeof(u32) * 256 * (size_t)nb, st));
  u64 *src = keys, *dst = tmp;
  for (int sh : shifts) {
    rs_hist_kernel<<<nb, RS_THREADS, 0, st>>>(src, n, sh, counts, nb);
    TC_NOTE_LAUNCH();
    TC_CUDA_TRY(cudaGetLastError());
    int rc = scan_exclusive<u32>(counts, counts, 256 * (int64_t)nb, st, (u32 *)nullptr);
    if (rc) return rc;
    rs_scatter_kernel<<<nb, RS_THREADS, 0, st>>>(src, dst, n, sh, counts, nb);
    TC_NOTE_LAUNCH();
    TC_CUDA_TRY(cudaGetLastError());
    std::swap(src, dst);
  }
  if (src != keys) TC_CUDA_TRY(cudaMemcpyAsync(keys, src, sizeof(u64) * n, cudaMemcpyDeviceToDevice, st));
  TC_CUDA_TRY(cudaFreeAsync(counts, st));
  return TRUST_TC_OK;
}

int radix_sort_u64(unsigned long long *keys, unsigned long long *tmp, int64_t n, const int *shifts, int nshifts,
                   cudaStream_t st) {
  return radix_sort(keys, tmp, n, std::vector<int>(shifts, shifts + nshifts), st);
}

static void push_digits(std::vector<int> &v, int lo, int bits) {
  for (int b = 0; b < bits; b += 8) v.push_back(lo + b);
}

static int bits_for(int64_t x) {  // bits needed to represent values in [0, x]
  int b = 1;
  while (b < 63 && ((int64_t)1 << b) <= x) ++b;
  return b;
}

// ------------------------------------------------------------------------------------------
// pipeline kernels
// ------------------------------------------------------------------------------------------
#define GRID_STRIDE(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void canon_kernel(const int32_t *__restrict__ pairs, int64_t np, int64_t id_bound, u64 *keys) {
  const u64 invalid = (u64)id_bound << 32;
  GRID_STRIDE(i, np) {
    int u = pairs[2 * i], v = pairs[2 * i + 1];
    bool ok = u != v && u >= 0 && v >= 0 && u < id_bound && v < id_bound;
    u64 a = (u64)(u32)min(u, v), b = (u64)(u32)max(u, v);
    keys[i] = ok ? ((a << 32) | b) : invalid;
  }
}

__global__ void unique_flags_kernel(const u64 *__restrict__ keys, int64_t n, int64_t id_bound, u32 *flags) {
  GRID_STRIDE(i, n) {
    u64 k = keys[i];
    flags[i] = ((int64_t)(k >> 32) < id_bound) && (i == 0 || keys[i - 1] != k);
  }
}

__global__ void compact_kernel(const u64 *__restrict__ keys, const u32 *__restrict__ flags,
                               const u32 *__restrict__ pos, int64_t n, u64 *out) {
  GRID_STRIDE(i, n) {
    if (flags[i]) out[pos[i]] = keys[i];
  }
}

__global__ void degree_kernel(const u64 *__restrict__ e, int64_t ne, u32 *deg) {
  GRID_STRIDE(i, ne) {
    u64 k = e[i];
    atomicAdd(&deg[k >> 32], 1u);
    atomicAdd(&deg[k & 0xffffffffu], 1u);
  }
}

__global__ void present_kernel(const u32 *__restrict__ deg, int64_t n, u32 *flags) {
  GRID_STRIDE(i, n) { flags[i] = deg[i] > 0; }
}

// orientation keys (degree, compacted id); cid = exclusive scan of the present flags
__global__ void vkey_kernel(const u32 *__restrict__ deg, const u32 *__restrict__ cid, int64_t n, u64 *vkeys) {
  GRID_STRIDE(x, n) {
    u32 d = deg[x];
    if (d) vkeys[cid[x]] = ((u64)d << 32) | cid[x];
  }
}

__global__ void position_kernel(const u64 *__restrict__ vkeys, int64_t n, u32 *pos) {
  GRID_STRIDE(p, n) { pos[vkeys[p] & 0xffffffffu] = (u32)p; }
}

__global__ void orient_kernel(u64 *e, int64_t ne, const u32 *__restrict__ cid, const u32 *__restrict__ pos,
                              u32 *od) {
  GRID_STRIDE(i, ne) {
    u64 k = e[i];
    u32 a = cid[k >> 32], b = cid[k & 0xffffffffu];
    bool a_first = pos[a] < pos[b];
    u32 s = a_first ? a : b, d = a_first ? b : a;
    e[i] = ((u64)s << 32) | d;
    atomicAdd(&od[s], 1u);
  }
}

__global__ void max_kernel(const u32 *__restrict__ x, int64_t n, u32 *mx) {
  u32 m = 0;
  GRID_STRIDE(i, n) { m = max(m, x[i]); }
  m = __reduce_max_sync(TC_FULL_MASK, m);
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

__global__ void renumber_key_kernel(const u32 *__restrict__ od, int64_t n, u32 dmax, u64 *vkeys) {
  GRID_STRIDE(c, n) { vkeys[c] = ((u64)(dmax - od[c]) << 32) | (u64)c; }
}

__global__ void relabel_kernel(u64 *e, int64_t ne, const u32 *__restrict__ newid) {
  GRID_STRIDE(i, ne) {
    u64 k = e[i];
    e[i] = ((u64)newid[k >> 32] << 32) | newid[k & 0xffffffffu];
  }
}

__global__ void csr_kernel(const u64 *__restrict__ arcs, int64_t ne, int64_t n, int64_t *beg, int32_t *adj) {
  GRID_STRIDE(i, ne) {
    u64 k = arcs[i];
    int64_t s = (int64_t)(k >> 32);
    adj[i] = (int32_t)(k & 0xffffffffu);
    int64_t prev = i == 0 ? -1 : (int64_t)(arcs[i - 1] >> 32);
    for (int64_t v = prev + 1; v <= s; ++v) beg[v] = i;
  }
}

__global__ void csr_tail_kernel(int64_t from, int64_t n, int64_t ne, int64_t *beg) {
  GRID_STRIDE(j, n + 1 - from) { beg[from + j] = ne; }
}

static int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32)); }

// ------------------------------------------------------------------------------------------
// host pipeline
// ------------------------------------------------------------------------------------------
struct DevBufs {
  std::vector<void *> ptrs;
  cudaStream_t st;
  ~DevBufs() {
    for (void *p : ptrs) cudaFreeAsync(p, st);
  }
  template <typename T>
  int get(T **p, int64_t count) {
    *p = nullptr;
    cudaError_t e = cudaMallocAsync((void **)p, sizeof(T) * (size_t)std::max<int64_t>(count, 1), st);
    if (e != cudaSuccess) return cuda_status(e);
    ptrs.push_back(*p);
    return TRUST_TC_OK;
  }
};

// seg_out[g] = compacted id of the first vertex at or after original id seg_in[g] (the present
// vertices before it), or n for seg_in[g] >= id_bound
__global__ void seg_map_kernel(const u32 *__restrict__ cid, int64_t id_bound, int64_t n,
                               const int64_t *__restrict__ seg_in, int64_t nseg, int64_t *seg_out) {
  GRID_STRIDE(g, nseg) {
    const int64_t x = seg_in[g];
    seg_out[g] = x >= id_bound ? n : (x <= 0 ? 0 : (int64_t)cid[x]);
  }
}

// keep_order: new ids are the compacted ids (original order kept, isolated vertices dropped)
// instead of the out-degree-descending renumbering; with d_seg_in / d_seg_out (nseg entries, on
// the device) the original-id boundaries of segments are mapped to the new ids.
int build_csr_device(const int32_t *d_pairs, int64_t np, int64_t id_bound, int64_t **d_beg_out,
                     int32_t **d_adj_out, int64_t *n_out, int64_t *m_out, cudaStream_t st, bool keep_order,
                     const int64_t *d_seg_in, int64_t nseg, int64_t *d_seg_out) {
  if (np < 0 || id_bound < 1 || id_bound >= ((int64_t)1 << 31)) return TRUST_TC_E_ARG;
  if (np >= ((int64_t)1 << 32) - 1) return TRUST_TC_E_TOO_LARGE;
  DevBufs B;
  B.st = st;
  int rc;
  u64 *keys, *tmp;
  u32 *flags, *pos;
  if ((rc = B.get(&keys, np)) || (rc = B.get(&tmp, np)) || (rc = B.get(&flags, np)) || (rc = B.get(&pos, np)))
    return rc;
  const int idb = bits_for(id_bound);  // covers the invalid marker id_bound
  // 1. canonical (min,max) keys, sorted; invalid pairs sort last
  canon_kernel<<<grid_for(np), 256, 0, st>>>(d_pairs, np, id_bound, keys);
  TC_NOTE_LAUNCH();
  std::vector<int> sh;
  push_digits(sh, 0, bits_for(id_bound - 1));
  push_digits(sh, 32, idb);
  if ((rc = radix_sort(keys, tmp, np, sh, st))) return rc;
  // 2. unique
  unique_flags_kernel<<<grid_for(np), 256, 0, st>>>(keys, np, id_bound, flags);
  TC_NOTE_LAUNCH();
  u32 nu32 = 0;
  if ((rc = scan_exclusive<u32>(flags, pos, np, st, &nu32))) return rc;
  const int64_t nu = nu32;
  u64 *e = tmp;  // unique edges live in tmp from here on
  compact_kernel<<<grid_for(np), 256, 0, st>>>(keys, flags, pos, np, e);
  TC_NOTE_LAUNCH();
  // 3. degrees and compacted ids (vertices without edges dropped)
  u32 *deg, *cid;
  if ((rc = B.get(&deg, id_bound)) || (rc = B.get(&cid, id_bound))) return rc;
  TC_CUDA_TRY(cudaMemsetAsync(deg, 0, sizeof(u32) * id_bound, st));
  degree_kernel<<<grid_for(nu), 256, 0, st>>>(e, nu, deg);
  TC_NOTE_LAUNCH();
  present_kernel<<<grid_for(id_bound), 256, 0, st>>>(deg, id_bound, cid);
  TC_NOTE_LAUNCH();
  u32 n32 = 0;
  if ((rc = scan_exclusive<u32>(cid, cid, id_bound, st, &n32))) return rc;
  const int64_t n = n32;
  // 4. orientation order (degree, compacted id) ascending
  u64 *vkeys, *vtmp;
  u32 *vpos, *od, *dmax;
  if ((rc = B.get(&vkeys, n)) || (rc = B.get(&vtmp, n)) || (rc = B.get(&vpos, n)) || (rc = B.get(&od, n)) || (rc = B.get(&dmax, 1))) return rc;
  vkey_kernel<<<grid_for(id_bound), 256, 0, st>>>(deg, cid, id_bound, vkeys);
  TC_NOTE_LAUNCH();
  TC_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(u32), st));
  max_kernel<<<grid_for(id_bound), 256, 0, st>>>(deg, id_bound, dmax);
  TC_NOTE_LAUNCH();
  u32 hdmax = 0;
  TC_CUDA_TRY(cudaMemcpyAsync(&hdmax, dmax, sizeof(u32), cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  sh.clear();
  push_digits(sh, 0, bits_for(std::max<int64_t>(n - 1, 1)));
  push_digits(sh, 32, bits_for(hdmax));
  if ((rc = radix_sort(vkeys, vtmp, n, sh, st))) return rc;
  position_kernel<<<grid_for(n), 256, 0, st>>>(vkeys, n, vpos);
  TC_NOTE_LAUNCH();
  // 5. orient each edge from the earlier to the later vertex of that order
  TC_CUDA_TRY(cudaMemsetAsync(od, 0, sizeof(u32) * n, st));
  orient_kernel<<<grid_for(nu), 256, 0, st>>>(e, nu, cid, vpos, od);
  TC_NOTE_LAUNCH();
  if (d_seg_in && nseg > 0) {
    seg_map_kernel<<<grid_for(nseg), 256, 0, st>>>(cid, id_bound, n, d_seg_in, nseg, d_seg_out);
    TC_NOTE_LAUNCH();
  }
  // 6. renumber: out-degree descending, ties by compacted id
  if (!keep_order) {
  TC_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(u32), st));
  max_kernel<<<grid_for(n), 256, 0, st>>>(od, n, dmax);
  TC_NOTE_LAUNCH();
  u32 hodmax = 0;
  TC_CUDA_TRY(cudaMemcpyAsync(&hodmax, dmax, sizeof(u32), cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  renumber_key_kernel<<<grid_for(n), 256, 0, st>>>(od, n, hodmax, vkeys);
  TC_NOTE_LAUNCH();
  sh.clear();
  push_digits(sh, 0, bits_for(std::max<int64_t>(n - 1, 1)));
  push_digits(sh, 32, bits_for(hodmax));
  if ((rc = radix_sort(vkeys, vtmp, n, sh, st))) return rc;
  position_kernel<<<grid_for(n), 256, 0, st>>>(vkeys, n, vpos);  // vpos = new id of compacted id
  TC_NOTE_LAUNCH();
  relabel_kernel<<<grid_for(nu), 256, 0, st>>>(e, nu, vpos);
  TC_NOTE_LAUNCH();
  }
  // 7. sort arcs by (source, target) and emit the CSR
  sh.clear();
  push_digits(sh, 0, bits_for(std::max<int64_t>(n - 1, 1)));
  push_digits(sh, 32, bits_for(std::max<int64_t>(n - 1, 1)));
  if ((rc = radix_sort(e, keys, nu, sh, st))) return rc;
  int64_t *beg = nullptr;
  int32_t *adj = nullptr;
  TC_CUDA_TRY(cudaMalloc((void **)&beg, sizeof(int64_t) * (size_t)(n + 1)));
  cudaError_t ea = cudaMalloc((void **)&adj, sizeof(int32_t) * (size_t)std::max<int64_t>(nu, 1));
  if (ea != cudaSuccess) {
    cudaFree(beg);
    return cuda_status(ea);
  }
  int64_t last_src = -1;
  if (nu > 0) {
    u64 last = 0;
    TC_CUDA_TRY(cudaMemcpyAsync(&last, e + nu - 1, sizeof(u64), cudaMemcpyDeviceToHost, st));
    TC_CUDA_TRY(cudaStreamSynchronize(st));
    last_src = (int64_t)(last >> 32);
    csr_kernel<<<grid_for(nu), 256, 0, st>>>(e, nu, n, beg, adj);
    TC_NOTE_LAUNCH();
  }
  csr_tail_kernel<<<grid_for(n + 1 - (last_src + 1)), 256, 0, st>>>(last_src + 1, n, nu, beg);
  TC_NOTE_LAUNCH();
  cudaError_t le = cudaGetLastError();
  cudaError_t se = cudaStreamSynchronize(st);
  if (le != cudaSuccess || se != cudaSuccess) {
    cudaFree(beg);
    cudaFree(adj);
    return cuda_status(le != cudaSuccess ? le : se);
  }
  *d_beg_out = beg;
  *d_adj_out = adj;
  *n_out = n;
  *m_out = nu;
  return TRUST_TC_OK;
}

}  // namespace tc

// ---- the n x n hash partition on the GPU ---------------------------------------------------
// Tile (i,j) of Preprocess/partition.cpp:72-121: the rows of vertices v = i (mod p) as local row
// v / p, restricted to entries w = j (mod p), stored as w / p; rows stay sorted.  A warp per
// row: one ballot per part and 32 entries, lane j keeps part j's count (pass 1) or cursor (pass 2).
__global__ void part_count_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                  int p, int64_t stride, int64_t *__restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    const int64_t b = beg[v], e = beg[v + 1];
    int64_t mine = 0;
    for (int64_t k0 = b; k0 < e; k0 += 32) {
      const bool valid = k0 + lane < e;
      const int jw = valid ? (int)(adj[k0 + lane] % p) : -1;
      for (int j = 0; j < p; ++j) {
        const unsigned msk = __ballot_sync(TC_FULL_MASK, jw == j);
        if (lane == j) mine += __popc(msk);
      }
    }
    if (lane < p) cnt[(int64_t)((v % p) * p + lane) * stride + v / p] = mine;
  }
}

__global__ void part_fill_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n, int p,
                                 int64_t stride, const int64_t *__restrict__ off, const int64_t *__restrict__ tbase,
                                 int32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = warp; v < n; v += nwarps) {
    const int64_t b = beg[v], e = beg[v + 1];
    if (b == e) continue;
    const int i = (int)(v % p);
    // lane j: where part j's entries of this row go (tile base + row offset)
    int64_t pos = lane < p ? tbase[i * p + lane] + off[(int64_t)(i * p + lane) * stride + v / p] : 0;
    for (int64_t k0 = b; k0 < e; k0 += 32) {
      const bool valid = k0 + lane < e;
      const int w = valid ? adj[k0 + lane] : 0;
      const int jw = valid ? w % p : -1;
      for (int j = 0; j < p; ++j) {
        const unsigned msk = __ballot_sync(TC_FULL_MASK, jw == j);
        const int64_t cur = __shfl_sync(TC_FULL_MASK, pos, j);
        if (jw == j) out[cur + __popc(msk & ((1u << lane) - 1u))] = w / p;
        if (lane == j) pos += __popc(msk);
      }
    }
  }
}

namespace tc {

int partition_device_to_host(const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, int p, PinnedTile *tiles) {
  if (n < 1 || m < 0 || p < 1 || p > 32) return TRUST_TC_E_ARG;
  cudaStream_t st = 0;
  const int64_t stride = (n + p - 1) / p + 1;  // rows of part 0, plus the end offset
  const size_t T = (size_t)p * p;
  int64_t *cnt = nullptr, *tbase = nullptr;
  int32_t *out = nullptr;
  for (size_t t = 0; t < T; ++t) tiles[t] = PinnedTile{};
  TC_CUDA_TRY(cudaMalloc((void **)&cnt, sizeof(int64_t) * T * (size_t)stride));
  auto done = [&](int rc) {
    cudaFree(cnt);
    cudaFree(tbase);
    cudaFree(out);
    return rc;
  };
  auto cu = [&](cudaError_t e) { return e == cudaSuccess ? TRUST_TC_OK : cuda_status(e); };
  int rc = cu(cudaMemsetAsync(cnt, 0, sizeof(int64_t) * T * (size_t)stride, st));
  if (rc) return done(rc);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, 152 * 64));
  part_count_kernel<<<blocks, 256, 0, st>>>(beg, adj, n, p, stride, cnt);
  TC_NOTE_LAUNCH();
  if ((rc = cu(cudaGetLastError()))) return done(rc);
  std::vector<int64_t> hbase(T + 1, 0);
  for (size_t t = 0; t < T; ++t) {
    const int i = (int)(t / p);
    const int64_t rows = n > i ? (n - i + p - 1) / p : 0;
    int64_t total = 0;
    if ((rc = scan_exclusive_i64(cnt + t * stride, cnt + t * stride, rows + 1, st, &total))) return done(rc);
    tiles[t].rows = rows;
    tiles[t].m = total;
    hbase[t + 1] = hbase[t] + total;
  }
  if (hbase[T] != m) return done(TRUST_TC_E_DEVICE);
  if ((rc = cu(cudaMalloc((void **)&tbase, sizeof(int64_t) * (T + 1))))) return done(rc);
  if ((rc = cu(cudaMalloc((void **)&out, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1))))) return done(rc);
  if ((rc = cu(cudaMemcpy(tbase, hbase.data(), sizeof(int64_t) * (T + 1), cudaMemcpyHostToDevice)))) return done(rc);
  part_fill_kernel<<<blocks, 256, 0, st>>>(beg, adj, n, p, stride, cnt, tbase, out);
  TC_NOTE_LAUNCH();
  if ((rc = cu(cudaGetLastError()))) return done(rc);
  for (size_t t = 0; t < T; ++t) {
    PinnedTile &x = tiles[t];
    if ((rc = cu(cudaMallocHost((void **)&x.beg, sizeof(int64_t) * (size_t)(x.rows + 1))))) break;
    if ((rc = cu(cudaMallocHost((void **)&x.adj, sizeof(int32_t) * (size_t)std::max<int64_t>(x.m, 1))))) break;
    if ((rc = cu(cudaMemcpy(x.beg, cnt + t * stride, sizeof(int64_t) * (size_t)(x.rows + 1), cudaMemcpyDeviceToHost))))
      break;
    if (x.m && (rc = cu(cudaMemcpy(x.adj, out + hbase[t], sizeof(int32_t) * (size_t)x.m, cudaMemcpyDeviceToHost))))
      break;
  }
  if (rc) {
    for (size_t t = 0; t < T; ++t) {
      cudaFreeHost(tiles[t].beg);
      cudaFreeHost(tiles[t].adj);
      tiles[t] = PinnedTile{};
    }
  }
  return done(rc);
}

}  // namespace tc

extern "C" int trust_tc_build_csr_device(trust_tc_ctx *ctx, const int32_t *d_pairs, int64_t npairs,
                                         int64_t id_bound, int64_t **d_begin, int32_t **d_adj, int64_t *n,
                                         int64_t *m) {
  if (!d_begin || !d_adj || !n || !m || (npairs > 0 && !d_pairs)) return TRUST_TC_E_ARG;
  *d_begin = nullptr;
  *d_adj = nullptr;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  return tc::build_csr_device(d_pairs, npairs, id_bound, d_begin, d_adj, n, m, (cudaStream_t)0, false, nullptr, 0,
                              nullptr);
}

extern "C" int trust_tc_build_batch_device(trust_tc_ctx *ctx, const int32_t *d_pairs, int64_t npairs,
                                           const int64_t *graph_vbeg, int64_t num_graphs, int64_t **d_begin,
                                           int32_t **d_adj, int64_t *n, int64_t *m, int64_t *graph_vbeg_out) {
  if (!d_begin || !d_adj || !n || !m || (npairs > 0 && !d_pairs) || num_graphs < 1 || !graph_vbeg ||
      !graph_vbeg_out || graph_vbeg[0] != 0)
    return TRUST_TC_E_ARG;
  for (int64_t g = 0; g < num_graphs; ++g)
    if (graph_vbeg[g] > graph_vbeg[g + 1]) return TRUST_TC_E_ARG;
  *d_begin = nullptr;
  *d_adj = nullptr;
  if (ctx) TC_CUDA_TRY(cudaSetDevice(ctx->device));
  const int64_t nseg = num_graphs + 1;
  int64_t *d_seg = nullptr;
  TC_CUDA_TRY(cudaMalloc((void **)&d_seg, sizeof(int64_t) * 2 * (size_t)nseg));
  cudaError_t e = cudaMemcpy(d_seg, graph_vbeg, sizeof(int64_t) * (size_t)nseg, cudaMemcpyHostToDevice);
  int rc = e == cudaSuccess ? TRUST_TC_OK : tc::cuda_status(e);
  if (!rc)
    rc = tc::build_csr_device(d_pairs, npairs, std::max<int64_t>(graph_vbeg[num_graphs], 1), d_begin, d_adj, n, m,
                              (cudaStream_t)0, true, d_seg, nseg, d_seg + nseg);
  if (!rc) {
    e = cudaMemcpy(graph_vbeg_out, d_seg + nseg, sizeof(int64_t) * (size_t)nseg, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = tc::cuda_status(e);
  }
  cudaFree(d_seg);
  return rc;
}

extern "C" void trust_tc_free_device(void *p) {
  if (p) cudaFree(p);
}

extern "C" int trust_tc_copy(void *dst, const void *src, size_t bytes) {
  if (!bytes) return TRUST_TC_OK;
  if (!dst || !src) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
  return TRUST_TC_OK;
}

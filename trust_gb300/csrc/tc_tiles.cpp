// tc_tiles.cpp — the n x n hash partition as a one-GPU tile loop.
//
// Preprocess/partition.cpp:72-121 splits an oriented CSR into parts x parts tiles: tile (i,j)
// holds the rows of vertices v with v % parts == i (local row v / parts) restricted to
// neighbours w with w % parts == j, stored as w / parts.  The reference then runs one MPI rank
// per (i,j,k) job (With-graph-partition/TC.cu:988-994): tables from part(i,j), arcs from
// part(i,k), probe lists from part(k,j).  Here all parts^3 jobs run on one GPU through the same
// persistent kernel, with the tiles kept in a device cache bounded by a byte budget so a graph
// larger than HBM streams its tiles in from host memory.
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <list>
#include <string>
#include <vector>

#include "tc_count.h"
#include "tc_internal.h"

namespace {

struct HostTile {
  int64_t *beg = nullptr;
  int32_t *adj = nullptr;
  int64_t rows = 0, m = 0;
};

struct DevTile {
  int64_t *beg = nullptr;
  int32_t *adj = nullptr;
  size_t bytes = 0;
  bool resident = false;
};

std::string tile_dir(const std::string &root, int i, int j) {
  return root + "/partition" + std::to_string(i) + "_" + std::to_string(j);
}

}  // namespace

extern "C" {

int trust_tc_partition_folder(const char *folder, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m,
                              int parts) {
  if (!folder || !beg || n < 0 || m < 0 || (m && !adj) || parts < 1 || parts > 64) return TRUST_TC_E_ARG;
  int rc = trust_tc_validate_csr(beg, adj, n, m, nullptr);
  if (rc) return rc;
  const int p = parts;
  std::vector<int64_t> rows(p), ents((size_t)p * p, 0);
  for (int i = 0; i < p; ++i) rows[i] = n > i ? (n - i + p - 1) / p : 0;
  for (int64_t v = 0; v < n; ++v)
    for (int64_t k = beg[v]; k < beg[v + 1]; ++k) ents[(size_t)(v % p) * p + adj[k] % p]++;
  std::vector<std::vector<int64_t>> tb((size_t)p * p);
  std::vector<std::vector<int32_t>> ta((size_t)p * p);
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) {
      tb[(size_t)i * p + j].assign((size_t)rows[i] + 1, 0);
      ta[(size_t)i * p + j].reserve((size_t)ents[(size_t)i * p + j]);
    }
  for (int64_t v = 0; v < n; ++v) {
    const int ii = (int)(v % p);
    const int64_t r = v / p;
    for (int64_t k = beg[v]; k < beg[v + 1]; ++k) ta[(size_t)ii * p + adj[k] % p].push_back(adj[k] / p);
    for (int j = 0; j < p; ++j) tb[(size_t)ii * p + j][(size_t)r + 1] = (int64_t)ta[(size_t)ii * p + j].size();
  }
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) {
      std::string d = tile_dir(folder, i, j);
      if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return TRUST_TC_E_IO;
      const auto &b = tb[(size_t)i * p + j];
      const auto &a = ta[(size_t)i * p + j];
      rc = trust_tc_save_folder(d.c_str(), b.data(), a.data(), rows[i], (int64_t)a.size());
      if (rc) return rc;
    }
  return TRUST_TC_OK;
}

}  // extern "C"

namespace tc {

// The (i,j,k) jobs over p x p host tiles (all p*p present, ht[i*p+j]), the tiles kept in a device
// cache with an LRU byte budget (0 = 80 % of the free memory at entry).  r->call_seconds covers
// the whole loop including the host-to-device tile copies.
int tile_loop(const std::vector<HostTile> &ht, int p, const trust_tc_opts &o, size_t budget_bytes,
              trust_tc_result *r) {
  int rc = TRUST_TC_OK;
  int64_t total_m = 0;
  for (const auto &t : ht) total_m += t.m;
  trust_tc_ctx ctx;
  rc = ctx_init(&ctx, o.device);
  if (rc) {
    ctx_release(&ctx);
    return rc;
  }
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const size_t budget = budget_bytes ? budget_bytes : free_b / 10 * 8;
  std::vector<DevTile> dt((size_t)p * p);
  std::list<int> lru;
  size_t used = 0;
  auto evict_one = [&](int keep0, int keep1, int keep2) -> bool {
    for (auto it = lru.rbegin(); it != lru.rend(); ++it) {
      int id = *it;
      if (id == keep0 || id == keep1 || id == keep2) continue;
      cudaFree(dt[id].beg);
      cudaFree(dt[id].adj);
      used -= dt[id].bytes;
      dt[id] = DevTile();
      lru.erase(std::next(it).base());
      return true;
    }
    return false;
  };
  uint64_t copied = 0;
  // per tile: rows strictly increasing (so duplicate-free), checked on its first copy; the
  // direction split of a job needs it of the job's table and probe tiles
  std::vector<signed char> increasing((size_t)p * p, -1);
  auto fetch = [&](int id, int k0, int k1, int k2) -> int {
    DevTile &d = dt[id];
    if (d.resident) {
      lru.remove(id);
      lru.push_front(id);
      return TRUST_TC_OK;
    }
    const HostTile &h = ht[id];
    size_t bytes = sizeof(int64_t) * (size_t)(h.rows + 1) + sizeof(int32_t) * (size_t)std::max<int64_t>(h.m, 1);
    while (used + bytes > budget && evict_one(k0, k1, k2)) {
    }
    cudaError_t e = cudaMalloc(&d.beg, sizeof(int64_t) * (size_t)(h.rows + 1));
    if (e == cudaSuccess) e = cudaMalloc(&d.adj, sizeof(int32_t) * (size_t)std::max<int64_t>(h.m, 1));
    if (e == cudaSuccess) e = cudaMemcpy(d.beg, h.beg, sizeof(int64_t) * (size_t)(h.rows + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && h.m) e = cudaMemcpy(d.adj, h.adj, sizeof(int32_t) * (size_t)h.m, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d.beg);
      cudaFree(d.adj);
      d = DevTile();
      return cuda_status(e);
    }
    copied += bytes;
    d.bytes = bytes;
    d.resident = true;
    used += bytes;
    lru.push_front(id);
    if (increasing[id] < 0) {
      bool inc = false;
      const int rc2 = rows_increasing(&ctx, d.beg, d.adj, h.rows, (cudaStream_t)o.stream, &inc);
      if (rc2) return rc2;
      increasing[id] = inc ? 1 : 0;
    }
    return TRUST_TC_OK;
  };
  uint64_t *cycles = r->vertex_cycles;
  memset(r, 0, sizeof *r);
  r->vertex_cycles = cycles;
  uint64_t total = 0;
  double tk = 0, tcount = 0;
  int64_t n_total = 0;
  for (int i = 0; i < p; ++i) n_total += ht[(size_t)i * p].rows;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, (cudaStream_t)o.stream);
  for (int i = 0; i < p && !rc; ++i)
    for (int j = 0; j < p && !rc; ++j)
      for (int k = 0; k < p && !rc; ++k) {
        const int A = i * p + j, Bt = i * p + k, C = k * p + j;
        if (ht[A].rows == 0 || ht[A].m == 0 || ht[Bt].m == 0) continue;
        if ((rc = fetch(A, A, Bt, C)) || (rc = fetch(Bt, A, Bt, C)) || (rc = fetch(C, A, Bt, C))) break;
        DevGraph3 g{};
        g.begA = dt[A].beg; g.adjA = dt[A].adj;
        g.begB = dt[Bt].beg; g.adjB = dt[Bt].adj;
        g.begC = dt[C].beg; g.adjC = dt[C].adj;
        g.rows = ht[A].rows;
        g.rowsC = ht[C].rows;
        g.mA = ht[A].m; g.mB = ht[Bt].m; g.mC = ht[C].m;
        // entries of tiles (i,j) and (k,j) are local ids of column class j, below the row count of
        // tile row class j (validated by the job's id check)
        g.boundA = g.boundC = ht[(size_t)j * p].rows;
        g.boundB = ht[C].rows;
        // a diagonal job (i,i,i) is one CSR: rows with one entry close no triangle there
        g.min_deg = (A == Bt && Bt == C) ? 2 : 1;
        g.split_ok = increasing[A] == 1 && increasing[C] == 1;
        trust_tc_result jr;
        memset(&jr, 0, sizeof jr);
        rc = count_device(&ctx, g, o, true, &jr);
        total += jr.triangles;
        r->wedges += jr.wedges;
        tk += jr.kernel_seconds;
        tcount += jr.count_seconds;
        r->max_out_degree = std::max(r->max_out_degree, jr.max_out_degree);
        r->direction_split += jr.direction_split;  // jobs counted with the split
        r->split_saving_ms += jr.split_saving_ms;
        for (int c = 0; c < TC_NUM_CLASSES; ++c) r->class_sizes[c] += jr.class_sizes[c];
      }
  cudaEventRecord(e1, (cudaStream_t)o.stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (auto &d : dt) {
    cudaFree(d.beg);
    cudaFree(d.adj);
  }
  ctx_release(&ctx);
  r->triangles = total;
  r->kernel_seconds = tk;
  r->count_seconds = tcount;
  r->call_seconds = ms * 1e-3;
  r->vertices = n_total;
  r->edges = total_m;
  (void)copied;
  return rc;
}

}  // namespace tc

extern "C" {

int trust_tc_count_tiles_device(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m, int parts,
                                size_t device_budget_bytes, const trust_tc_opts *opts, trust_tc_result *r) {
  if (!d_begin || (m > 0 && !d_adj) || n < 1 || m < 0 || n >= ((int64_t)1 << 31) || m >= ((int64_t)1 << 31) ||
      !r || parts < 1 || parts > 32)
    return TRUST_TC_E_ARG;
  trust_tc_opts o;
  if (opts) o = *opts; else trust_tc_opts_init(&o);
  if (o.row_begin || o.row_end) return TRUST_TC_E_UNSUPPORTED;  // row ranges: single-graph calls only
  int rc = TRUST_TC_OK;
  {  // validate the whole CSR before the partition reads it
    trust_tc_ctx ctx;
    rc = tc::ctx_init(&ctx, o.device);
    if (!rc) {
      cudaError_t e = cudaMemset(ctx.d_ctl, 0, sizeof(TcControl));
      rc = e == cudaSuccess ? tc::launch_check(d_begin, d_adj, n, m, n, 1, ctx.d_ctl, ctx.num_sms, 0)
                            : tc::cuda_status(e);
      if (!rc) {
        e = cudaMemcpy(ctx.h_ctl, ctx.d_ctl, sizeof(TcControl), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = tc::cuda_status(e);
      }
      if (!rc) {
        const int st = ctx.h_ctl->status;
        if (st & TC_DEV_BAD_OFFSETS) rc = TRUST_TC_E_OFFSETS;
        else if (st & TC_DEV_TOO_LARGE) rc = TRUST_TC_E_TOO_LARGE;
        else if (st & TC_DEV_BAD_IDS) rc = TRUST_TC_E_IDS;
      }
    }
    tc::ctx_release(&ctx);
    if (rc) return rc;
  }
  const int p = parts;
  std::vector<tc::PinnedTile> pt((size_t)p * p);
  rc = tc::partition_device_to_host(d_begin, d_adj, n, m, p, pt.data());
  if (rc) return rc;
  std::vector<HostTile> ht((size_t)p * p);
  for (size_t t = 0; t < pt.size(); ++t) {
    ht[t].beg = pt[t].beg;
    ht[t].adj = pt[t].adj;
    ht[t].rows = pt[t].rows;
    ht[t].m = pt[t].m;
  }
  rc = tc::tile_loop(ht, p, o, device_budget_bytes, r);
  for (auto &t : pt) {
    cudaFreeHost(t.beg);
    cudaFreeHost(t.adj);
  }
  return rc;
}

int trust_tc_count_partitioned(const char *folder, int parts, const trust_tc_opts *opts, trust_tc_result *r) {
  if (!folder || !r || parts < 1 || parts > 64) return TRUST_TC_E_ARG;
  trust_tc_opts o;
  if (opts) o = *opts; else trust_tc_opts_init(&o);
  if (o.row_begin || o.row_end) return TRUST_TC_E_UNSUPPORTED;  // row ranges: single-graph calls only
  const int p = parts;
  std::vector<HostTile> ht((size_t)p * p);
  int rc = TRUST_TC_OK;
  for (int i = 0; i < p && !rc; ++i)
    for (int j = 0; j < p && !rc; ++j) {
      HostTile &t = ht[(size_t)i * p + j];
      rc = trust_tc_load_folder(tile_dir(folder, i, j).c_str(), &t.beg, &t.adj, &t.rows, &t.m);
    }
  for (int i = 0; i < p && !rc; ++i)
    for (int j = 1; j < p && !rc; ++j)
      if (ht[(size_t)i * p + j].rows != ht[(size_t)i * p].rows) rc = TRUST_TC_E_FORMAT;
  if (!rc) rc = tc::tile_loop(ht, p, o, 0, r);
  for (auto &t : ht) {
    free(t.beg);
    free(t.adj);
  }
  return rc;
}

}  // extern "C"

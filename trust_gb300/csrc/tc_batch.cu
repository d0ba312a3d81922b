// tc_batch.cu — many graphs counted by one CUDA-graph launch.
//
// The reference counts one graph per run (Without-graph-partition/mpi_main.cpp:75-119): a batch
// of thousands of small graphs through it is a loop of runs, each paying its own launches and
// host synchronisations.  Here a batch is the disjoint union of its graphs in one oriented CSR
// (trust_tc_build_batch_device keeps every graph a contiguous row range), and one captured CUDA
// graph does the whole job on the device: validation, a classification of every row by (size
// class of its graph, degree class) with each size class's own warp-class bound, list offsets
// computed on the device (degree class major, so every degree class is one list over all size
// classes), one persistent counting kernel over all of them, and the readback of the per-graph
// counts.  Hits are attributed to graphs inside the counting kernel (CountArgs graph_of /
// graph_counts).  One launch instead of one per size class: measured on GB300 for the 4096-graph
// workload, 14.6 ms for the union in one launch against 16.8 ms for four autotuned per-class
// launches (the classes' kernels ran one after another, each draining to its own tail).  The
// autotuner times the whole job for each candidate (threads per CTA, warp-class bound, queue
// chunk), then each size class's warp-class bound on its own.
#include <string.h>

#include <algorithm>
#include <vector>

#include "tc_count.h"
#include "tc_internal.h"

using namespace tc;

namespace {

// size classes by vertex count: [0, 512), [512, 4096), [4096, 32768), [32768, ...)
constexpr int64_t SC_LIMIT[TC_BATCH_CLASSES - 1] = {512, 4096, 32768};
constexpr int CTA_MAX = 4096;  // CTA-class bound of every size class (hub rows above it spill)

int size_class_of(int64_t nv) {
  int s = 0;
  while (s < TC_BATCH_CLASSES - 1 && nv >= SC_LIMIT[s]) ++s;
  return s;
}

int ceil_log2(int64_t x) {
  int l = 0;
  while (((int64_t)1 << l) < x) ++l;
  return l;
}

// graph of every row: the last g with vbeg[g] <= v (empty graphs resolve to the next non-empty)
__global__ void graph_of_kernel(const int64_t *__restrict__ vbeg, int64_t G, int64_t n, int *__restrict__ graph_of) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = G - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) / 2;
      if (vbeg[mid] <= v) lo = mid; else hi = mid - 1;
    }
    graph_of[v] = (int)lo;
  }
}

// Per size class: the largest out-degree; and whether any arc leaves its graph (bad = 1).
__global__ void batch_scan_kernel(const int64_t *__restrict__ beg, const int32_t *__restrict__ adj, int64_t n,
                                  const int *__restrict__ graph_of, const unsigned char *__restrict__ graph_sc,
                                  int *__restrict__ maxdeg, int *__restrict__ bad) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int cross = 0;
  for (int64_t v = warp; v < n; v += nwarps) {
    const int64_t b = beg[v], e = beg[v + 1];
    const int g = graph_of[v];
    if (lane == 0) atomicMax(maxdeg + graph_sc[g], (int)(e - b));
    for (int64_t i = b + lane; i < e; i += 32) {
      const int u = adj[i];
      cross |= (u < 0 || (int64_t)u >= n) ? 1 : (graph_of[u] != g);
    }
  }
  cross = __reduce_or_sync(TC_FULL_MASK, cross);
  if (lane == 0 && cross) atomicOr(bad, 1);
}

}  // namespace

struct trust_tc_batch {
  trust_tc_ctx *ctx = nullptr;
  const int64_t *beg = nullptr;
  const int32_t *adj = nullptr;
  int64_t n = 0, m = 0, G = 0;
  int64_t graphs[TC_BATCH_CLASSES] = {}, vertices[TC_BATCH_CLASSES] = {};
  int maxdeg[TC_BATCH_CLASSES] = {};
  trust_tc_batch_class cfg[TC_BATCH_CLASSES];
  // the resolved counting launch (one for every size class)
  int threads = 256, chunk = 8, blocks = 0, warp_slots = 0, long_cap = 0;
  size_t smem = 0;
  int64_t *d_vbeg = nullptr;
  int *d_graph_of = nullptr;
  unsigned char *d_graph_sc = nullptr;
  unsigned long long *d_counts = nullptr, *h_counts = nullptr;  // h_counts pinned
  // one per size class, then the combined block of the single counting launch; h_ctl pinned
  TcControl *d_ctl = nullptr, *h_ctl = nullptr;
  int *d_lists = nullptr;
  int *d_huge = nullptr;
  int huge_log2 = 0, huge_blocks = 0;
  int2 *d_long = nullptr;
  size_t long_bytes = 0;
  cudaStream_t st = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels_per_run = 0;
  cudaEvent_t ev[2 + 2 * TC_BATCH_CLASSES] = {};
};

namespace {

void batch_release(trust_tc_batch *b) {
  if (b->ctx) cudaSetDevice(b->ctx->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  cudaFree(b->d_vbeg);
  cudaFree(b->d_graph_of);
  cudaFree(b->d_graph_sc);
  cudaFree(b->d_counts);
  cudaFreeHost(b->h_counts);
  cudaFree(b->d_ctl);
  cudaFreeHost(b->h_ctl);
  cudaFree(b->d_lists);
  cudaFree(b->d_huge);
  cudaFree(b->d_long);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->st) cudaStreamDestroy(b->st);
}

int check_class_cfg(const trust_tc_batch_class &c) {
  if (c.threads_per_block < 64 || c.threads_per_block > 1024 || c.threads_per_block % 32) return TRUST_TC_E_ARG;
  if (c.warp_max_degree < 32 || c.warp_max_degree > 1024) return TRUST_TC_E_ARG;
  if (c.chunk < 1 || c.chunk > 64) return TRUST_TC_E_ARG;
  return TRUST_TC_OK;
}

// The counting launch under the current configuration: one CTA size and queue chunk for every size
// class (those of the largest size class present; the autotuner keeps them equal), warp tables for
// the largest warp-class bound, a CTA table for the largest row a CTA takes, and scratch sized
// for it.  Not a stream operation: done before any capture.
constexpr int NCTL = TC_BATCH_CLASSES + 1;  // control blocks: per size class, then the combined one

int batch_prepare(trust_tc_batch *b) {
  const int num_sms = b->ctx->num_sms;
  int top = 0;
  for (int s = 0; s < TC_BATCH_CLASSES; ++s)
    if (b->graphs[s]) top = s;
  b->threads = b->cfg[top].threads_per_block;
  b->chunk = b->cfg[top].chunk;
  const int warps = b->threads / 32;
  int slots = 0, dcta = 1;
  bool cta = false;
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) {
    if (!b->graphs[s]) continue;
    const trust_tc_batch_class &c = b->cfg[s];
    slots = std::max(slots, 1 << std::max(ceil_log2(2 * (int64_t)std::min(c.warp_max_degree, std::max(b->maxdeg[s], 1))), 7));
    if (b->maxdeg[s] > c.warp_max_degree) {
      cta = true;
      dcta = std::max(dcta, std::min(b->maxdeg[s], CTA_MAX));
    }
  }
  b->warp_slots = std::max(slots, 128);
  size_t sm = (size_t)4 * b->warp_slots * warps;
  if (cta) sm = std::max(sm, (size_t)4 << std::max(ceil_log2(2 * (int64_t)dcta), 6));
  if (sm > (size_t)b->ctx->max_smem_optin) return TRUST_TC_E_ARG;
  b->smem = sm;
  int per_sm = 0;
  int rc = count_kernel_occupancy(true, b->threads, sm, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return TRUST_TC_E_ARG;
  b->blocks = num_sms * per_sm;
  b->long_cap = dcta;
  if ((rc = set_count_kernel_carveout(true, b->threads, sm, per_sm))) return rc;
  const size_t long_need = sizeof(int2) * (size_t)b->long_cap * (size_t)b->blocks;
  if (long_need > b->long_bytes) {
    cudaFree(b->d_long);
    b->d_long = nullptr;
    b->long_bytes = 0;
    TC_CUDA_TRY(cudaMalloc((void **)&b->d_long, long_need));
    b->long_bytes = long_need;
  }
  return TRUST_TC_OK;
}

// The whole job on stream st (captured, or run directly with per-class events when timed).
int batch_enqueue(trust_tc_batch *b, cudaStream_t st, bool timed) {
  const int num_sms = b->ctx->num_sms;
  TC_CUDA_TRY(cudaMemsetAsync(b->d_ctl, 0, sizeof(TcControl) * NCTL, st));
  TC_CUDA_TRY(cudaMemsetAsync(b->d_counts, 0, sizeof(unsigned long long) * (size_t)b->G, st));
  int rc = launch_check(b->beg, b->adj, b->n, b->m, b->n, 1, b->d_ctl, num_sms, st);
  if (rc) return rc;
  BatchThresholds th;
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) {
    th.warp_max[s] = b->cfg[s].warp_max_degree;
    th.cta_max[s] = CTA_MAX;
  }
  if ((rc = launch_batch_classify(0, b->beg, b->n, b->d_graph_of, b->d_graph_sc, th, b->d_ctl, b->d_lists, num_sms,
                                  st)))
    return rc;
  if ((rc = launch_batch_offsets(b->d_ctl, TC_BATCH_CLASSES, st))) return rc;
  if ((rc = launch_batch_classify(1, b->beg, b->n, b->d_graph_of, b->d_graph_sc, th, b->d_ctl, b->d_lists, num_sms,
                                  st)))
    return rc;
  CountArgs a{};
  a.begA = a.begB = a.begC = b->beg;
  a.adjA = a.adjB = a.adjC = b->adj;
  a.rows = b->n;
  a.lists = b->d_lists;
  a.ctl = b->d_ctl + TC_BATCH_CLASSES;  // the combined lists of every size class
  a.huge_tables = b->d_huge;
  a.huge_log2 = b->huge_log2;
  a.huge_blocks = std::min(b->huge_blocks, b->blocks);
  a.warp_slots = b->warp_slots;
  a.chunk = b->chunk;
  a.long_rows = b->d_long;
  a.long_cap = b->long_cap;
  a.graph_of = b->d_graph_of;
  a.graph_counts = b->d_counts;
  a.dev_off = 1;
  if (timed) TC_CUDA_TRY(cudaEventRecord(b->ev[2], st));
  if ((rc = launch_count(true, a, b->blocks, b->threads, b->smem, st))) return rc;
  if (timed) TC_CUDA_TRY(cudaEventRecord(b->ev[3], st));
  TC_CUDA_TRY(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(TcControl) * NCTL, cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaMemcpyAsync(b->h_counts, b->d_counts, sizeof(unsigned long long) * (size_t)b->G,
                              cudaMemcpyDeviceToHost, st));
  return TRUST_TC_OK;
}

int batch_status(const trust_tc_batch *b) {
  const int st0 = b->h_ctl[0].status;
  if (st0 & TC_DEV_BAD_OFFSETS) return TRUST_TC_E_OFFSETS;
  if (st0 & TC_DEV_TOO_LARGE) return TRUST_TC_E_TOO_LARGE;
  if (st0 & TC_DEV_BAD_IDS) return TRUST_TC_E_IDS;
  for (int s = 0; s < NCTL; ++s)
    if (b->h_ctl[s].status & TC_DEV_TABLE_FULL) return TRUST_TC_E_DEVICE;
  return TRUST_TC_OK;
}

// Capture the job into a CUDA graph (replacing the previous one).  The kernels captured are not
// launches yet: the launch counter is corrected here and advanced by every run instead.
int batch_build_graph(trust_tc_batch *b) {
  int rc = batch_prepare(b);
  if (rc) return rc;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  const uint64_t before = trust_tc_kernel_launches();
  TC_CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  rc = batch_enqueue(b, b->st, false);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->st, &graph);
  const uint64_t captured = trust_tc_kernel_launches() - before;
  note_launch(0 - captured);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  TC_CUDA_TRY(e);
  e = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  TC_CUDA_TRY(e);
  b->kernels_per_run = captured;
  return TRUST_TC_OK;
}

}  // namespace

extern "C" {

int trust_tc_batch_create(trust_tc_ctx *ctx, const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                          const int64_t *graph_vbeg, int64_t num_graphs, trust_tc_batch **out) {
  if (!ctx || !out || !graph_vbeg || num_graphs < 1 || num_graphs >= ((int64_t)1 << 31) || n < 1 || m < 0 ||
      n >= ((int64_t)1 << 31) || m >= ((int64_t)1 << 31) || !d_begin || (m > 0 && !d_adj))
    return TRUST_TC_E_ARG;
  *out = nullptr;
  if (graph_vbeg[0] != 0 || graph_vbeg[num_graphs] != n) return TRUST_TC_E_ARG;
  for (int64_t g = 0; g < num_graphs; ++g)
    if (graph_vbeg[g] > graph_vbeg[g + 1]) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaSetDevice(ctx->device));
  trust_tc_batch *b = new trust_tc_batch();
  b->ctx = ctx;
  b->beg = d_begin;
  b->adj = d_adj;
  b->n = n;
  b->m = m;
  b->G = num_graphs;
  std::vector<unsigned char> sc((size_t)num_graphs);
  for (int64_t g = 0; g < num_graphs; ++g) {
    const int64_t nv = graph_vbeg[g + 1] - graph_vbeg[g];
    sc[(size_t)g] = (unsigned char)size_class_of(nv);
    b->graphs[sc[(size_t)g]] += 1;
    b->vertices[sc[(size_t)g]] += nv;
  }
  for (auto &c : b->cfg) c = trust_tc_batch_class{256, 128, 8};
  auto fail = [&](int rc) {
    batch_release(b);
    delete b;
    return rc;
  };
  auto cu = [&](cudaError_t e) { return e == cudaSuccess ? TRUST_TC_OK : cuda_status(e); };
  int rc = TRUST_TC_OK;
  if ((rc = cu(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking)))) return fail(rc);
  for (auto &e : b->ev)
    if ((rc = cu(cudaEventCreate(&e)))) return fail(rc);
  const size_t G = (size_t)num_graphs;
  if ((rc = cu(cudaMalloc((void **)&b->d_vbeg, sizeof(int64_t) * (G + 1))))) return fail(rc);
  if ((rc = cu(cudaMalloc((void **)&b->d_graph_of, sizeof(int) * (size_t)n)))) return fail(rc);
  if ((rc = cu(cudaMalloc((void **)&b->d_graph_sc, G)))) return fail(rc);
  if ((rc = cu(cudaMalloc((void **)&b->d_counts, sizeof(unsigned long long) * G)))) return fail(rc);
  if ((rc = cu(cudaMallocHost((void **)&b->h_counts, sizeof(unsigned long long) * G)))) return fail(rc);
  if ((rc = cu(cudaMalloc((void **)&b->d_ctl, sizeof(TcControl) * NCTL)))) return fail(rc);
  if ((rc = cu(cudaMallocHost((void **)&b->h_ctl, sizeof(TcControl) * NCTL)))) return fail(rc);
  memset(b->h_ctl, 0, sizeof(TcControl) * NCTL);
  if ((rc = cu(cudaMalloc((void **)&b->d_lists, sizeof(int) * (size_t)n)))) return fail(rc);
  if ((rc = cu(cudaMemcpy(b->d_vbeg, graph_vbeg, sizeof(int64_t) * (G + 1), cudaMemcpyHostToDevice)))) return fail(rc);
  if ((rc = cu(cudaMemcpy(b->d_graph_sc, sc.data(), G, cudaMemcpyHostToDevice)))) return fail(rc);
  // validation of the union (offsets, ids, row lengths), then graph ids and the per-class scan
  if ((rc = cu(cudaMemsetAsync(b->d_ctl, 0, sizeof(TcControl) * NCTL, b->st)))) return fail(rc);
  if ((rc = launch_check(d_begin, d_adj, n, m, n, 1, b->d_ctl, ctx->num_sms, b->st))) return fail(rc);
  if ((rc = cu(cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(TcControl) * NCTL, cudaMemcpyDeviceToHost,
                               b->st))))
    return fail(rc);
  if ((rc = cu(cudaStreamSynchronize(b->st)))) return fail(rc);
  if ((rc = batch_status(b))) return fail(rc);
  const int vb = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 16));
  graph_of_kernel<<<vb, 256, 0, b->st>>>(b->d_vbeg, num_graphs, n, b->d_graph_of);
  note_launch();
  int *d_scan = nullptr;  // maxdeg[TC_BATCH_CLASSES], bad
  if ((rc = cu(cudaMalloc((void **)&d_scan, sizeof(int) * (TC_BATCH_CLASSES + 1))))) return fail(rc);
  cudaError_t e = cudaMemsetAsync(d_scan, 0, sizeof(int) * (TC_BATCH_CLASSES + 1), b->st);
  if (e == cudaSuccess) {
    batch_scan_kernel<<<(int)std::min<int64_t>((n * 32 + 255) / 256, (int64_t)ctx->num_sms * 16), 256, 0, b->st>>>(
        d_begin, d_adj, n, b->d_graph_of, b->d_graph_sc, d_scan, d_scan + TC_BATCH_CLASSES);
    note_launch();
    e = cudaGetLastError();
  }
  int hs[TC_BATCH_CLASSES + 1] = {};
  if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d_scan, sizeof hs, cudaMemcpyDeviceToHost, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  cudaFree(d_scan);
  if ((rc = cu(e))) return fail(rc);
  if (hs[TC_BATCH_CLASSES]) return fail(TRUST_TC_E_IDS);  // an arc leaves its graph
  int dmax = 0;
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) {
    b->maxdeg[s] = hs[s];
    dmax = std::max(dmax, hs[s]);
  }
  if (dmax > CTA_MAX) {  // hub rows beyond the CTA table: global spill tables, 2 GiB at most
    b->huge_log2 = ceil_log2(2 * (int64_t)dmax);
    const size_t per = (size_t)4 << b->huge_log2;
    b->huge_blocks = (int)std::max<size_t>(1, std::min<size_t>(((size_t)1 << 31) / per, (size_t)ctx->num_sms * 16));
    if ((rc = cu(cudaMalloc((void **)&b->d_huge, per * (size_t)b->huge_blocks)))) return fail(rc);
  }
  if ((rc = batch_build_graph(b))) return fail(rc);
  *out = b;
  return TRUST_TC_OK;
}

void trust_tc_batch_destroy(trust_tc_batch *b) {
  if (!b) return;
  batch_release(b);
  delete b;
}

int trust_tc_batch_info(const trust_tc_batch *b, int64_t *graphs, int64_t *vertices, int32_t *max_out_degree) {
  if (!b) return TRUST_TC_E_ARG;
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) {
    if (graphs) graphs[s] = b->graphs[s];
    if (vertices) vertices[s] = b->vertices[s];
    if (max_out_degree) max_out_degree[s] = b->maxdeg[s];
  }
  return TRUST_TC_OK;
}

int trust_tc_batch_get_class(const trust_tc_batch *b, int size_class, trust_tc_batch_class *cfg) {
  if (!b || !cfg || size_class < 0 || size_class >= TC_BATCH_CLASSES) return TRUST_TC_E_ARG;
  *cfg = b->cfg[size_class];
  return TRUST_TC_OK;
}

int trust_tc_batch_set_class(trust_tc_batch *b, int size_class, const trust_tc_batch_class *cfg) {
  if (!b || !cfg || size_class < 0 || size_class >= TC_BATCH_CLASSES) return TRUST_TC_E_ARG;
  int rc = check_class_cfg(*cfg);
  if (rc) return rc;
  TC_CUDA_TRY(cudaSetDevice(b->ctx->device));
  const trust_tc_batch_class old = b->cfg[size_class];
  b->cfg[size_class] = *cfg;
  rc = batch_build_graph(b);
  if (rc) {
    b->cfg[size_class] = old;
    batch_build_graph(b);
  }
  return rc;
}

int trust_tc_batch_run(trust_tc_batch *b, void *stream, uint64_t *counts, trust_tc_result *r) {
  if (!b) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaSetDevice(b->ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  TC_CUDA_TRY(cudaEventRecord(b->ev[0], st));
  TC_CUDA_TRY(cudaGraphLaunch(b->exec, st));
  TC_CUDA_TRY(cudaEventRecord(b->ev[1], st));
  TC_CUDA_TRY(cudaEventSynchronize(b->ev[1]));
  note_launch(b->kernels_per_run);
  int rc = batch_status(b);
  if (rc) return rc;
  if (counts) memcpy(counts, b->h_counts, sizeof(uint64_t) * (size_t)b->G);
  if (r) {
    float ms = 0;
    TC_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
    memset(r, 0, sizeof *r);
    for (int s = 0; s < NCTL; ++s) {
      r->triangles += b->h_ctl[s].count;
      r->wedges += (int64_t)b->h_ctl[s].wedges;
    }
    for (int c = 0; c < TC_NUM_CLASSES; ++c) r->class_sizes[c] = b->h_ctl[TC_BATCH_CLASSES].class_count[c];
    r->kernel_seconds = r->count_seconds = r->call_seconds = ms * 1e-3;
    r->vertices = b->n;
    r->edges = b->m;
    r->max_out_degree = b->h_ctl[0].max_out_degree;
  }
  return TRUST_TC_OK;
}

int trust_tc_batch_autotune(trust_tc_batch *b, int repeats, double *best_ms) {
  if (!b || repeats < 1) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaSetDevice(b->ctx->device));
  static const int kThreads[] = {128, 256, 512, 1024};
  static const int kWarpMax[] = {64, 128};
  static const int kChunk[] = {2, 4, 8, 16};
  trust_tc_batch_class best[TC_BATCH_CLASSES];
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) best[s] = b->cfg[s];
  double best_t = 1e300;
  // the counting kernel's time under the current configuration (fastest of `repeats` runs);
  // TRUST_TC_E_ARG when it does not fit (shared memory)
  auto time_job = [&](double *ms_out) -> int {
    int rc = batch_prepare(b);
    if (rc) return rc;
    double t = 1e300;
    for (int k = 0; k < repeats; ++k) {
      if ((rc = batch_enqueue(b, b->st, true))) return rc;
      TC_CUDA_TRY(cudaStreamSynchronize(b->st));
      if ((rc = batch_status(b))) return rc;
      float ms = 0;
      TC_CUDA_TRY(cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]));
      t = std::min(t, (double)ms);
    }
    *ms_out = t;
    return TRUST_TC_OK;
  };
  // every size class the same (threads, warp bound, chunk), then each class's warp bound alone
  for (int t : kThreads)
    for (int w : kWarpMax)
      for (int ch : kChunk) {
        for (auto &c : b->cfg) c = trust_tc_batch_class{t, w, ch};
        double ms = 0;
        int rc = time_job(&ms);
        if (rc == TRUST_TC_E_ARG) continue;  // not a candidate
        if (rc) return rc;
        if (ms < best_t) {
          best_t = ms;
          for (int s = 0; s < TC_BATCH_CLASSES; ++s) best[s] = b->cfg[s];
        }
      }
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) {
    if (!b->graphs[s]) continue;
    for (int w : kWarpMax) {
      if (w == best[s].warp_max_degree) continue;
      for (int k = 0; k < TC_BATCH_CLASSES; ++k) b->cfg[k] = best[k];
      b->cfg[s].warp_max_degree = w;
      double ms = 0;
      int rc = time_job(&ms);
      if (rc == TRUST_TC_E_ARG) continue;
      if (rc) return rc;
      if (ms < best_t) {
        best_t = ms;
        best[s] = b->cfg[s];
      }
    }
  }
  for (int s = 0; s < TC_BATCH_CLASSES; ++s) b->cfg[s] = best[s];
  if (best_ms) *best_ms = best_t;
  return batch_build_graph(b);
}

}  // extern "C"

// tc_api.cpp — C ABI of the counter: contexts, validation, folder I/O, the count call.
//
// Host operator that replaces Triangle_count (Without-graph-partition/TC.cu:602-731): it loads
// the CSR (graph::graph, Without-graph-partition/graph.hpp:18-67), checks it, copies it to the
// device, classifies vertices (the degree split of TC.cu:632, generalised), launches the
// persistent counting kernel and reads the u64 count back.  Unlike the reference it validates
// input, never exits, reuses device scratch across calls through a context, and times the
// kernels with CUDA events instead of process CPU time (TC.cu:686-692).
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "tc_count.h"
#include "tc_internal.h"
#include "tc_model.h"

namespace tc {

static thread_local char g_cuda_err[256] = "";
static std::atomic<uint64_t> g_kernel_launches{0};

void note_launch(uint64_t k) { g_kernel_launches.fetch_add(k, std::memory_order_relaxed); }

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TRUST_TC_OK;
  snprintf(g_cuda_err, sizeof g_cuda_err, "%s (%s)", cudaGetErrorString(e), cudaGetErrorName(e));
  if (e == cudaErrorMemoryAllocation) return TRUST_TC_E_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TRUST_TC_E_NO_DEVICE;
  return TRUST_TC_E_CUDA;
}

int ctx_init(trust_tc_ctx *c, int device) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    if (e != cudaSuccess) cuda_status(e);
    return TRUST_TC_E_NO_DEVICE;
  }
  if (device < 0) TC_CUDA_TRY(cudaGetDevice(&device));
  if (device >= ndev) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaSetDevice(device));
  c->device = device;
  TC_CUDA_TRY(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  TC_CUDA_TRY(cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  TC_CUDA_TRY(cudaDeviceGetAttribute(&c->clock_khz, cudaDevAttrClockRate, device));
  TC_CUDA_TRY(cudaMalloc(&c->d_ctl, sizeof(TcControl)));
  TC_CUDA_TRY(cudaMallocHost(&c->h_ctl, sizeof(TcControl)));
  TC_CUDA_TRY(cudaMallocHost(&c->h_plans, TC_PLAN_WORDS * sizeof(unsigned long long)));
  for (auto &ev : c->ev) TC_CUDA_TRY(cudaEventCreate(&ev));
  for (auto &ev : c->ev_split) TC_CUDA_TRY(cudaEventCreate(&ev));
  for (auto &sl : c->staged) TC_CUDA_TRY(cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming));
  TC_CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  return TRUST_TC_OK;
}

void ctx_release(trust_tc_ctx *c) {
  if (c->device >= 0) cudaSetDevice(c->device);
  if (c->sub) {
    ctx_release(c->sub);
    delete c->sub;
    c->sub = nullptr;
  }
  if (c->sub_stream) {
    cudaStreamSynchronize(c->sub_stream);
    cudaStreamDestroy(c->sub_stream);
    c->sub_stream = nullptr;
  }
  if (c->copy_stream) {  // staged copies still in flight finish before their buffers go
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
    c->copy_stream = nullptr;
  }
  for (auto &sl : c->staged) {
    cudaFree(sl.d_beg);
    cudaFree(sl.d_adj);
    if (sl.ready) cudaEventDestroy(sl.ready);
    sl = trust_tc_ctx::Staged();
  }
  cudaFree(c->d_ctl);
  cudaFreeHost(c->h_ctl);
  cudaFreeHost(c->h_plans);
  cudaFree(c->d_lists);
  cudaFree(c->d_huge);
  cudaFree(c->d_long);
  cudaFree(c->d_split_cnt);
  cudaFree(c->d_dec);
  cudaFree(c->d_pred);
  cudaFree(c->d_model);
  cudaFree(c->d_sort);
  cudaFree(c->d_split_wsum);
  cudaFree(c->d_split_plans);
  cudaFree(c->d_sched_long);
  cudaFree(c->d_split_pairs);
  cudaFree(c->d_split_beg);
  cudaFree(c->d_split_cbase);
  cudaFree(c->d_split_cbeg);
  cudaFree(c->d_split_rowmap);
  cudaFree(c->d_split_adj);
  cudaFree(c->d_beg);
  cudaFree(c->d_adj);
  for (auto &ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto &ev : c->ev_split)
    if (ev) cudaEventDestroy(ev);
  *c = trust_tc_ctx();
}

// Grow a device buffer to at least `bytes` (contents are not kept).
int ensure(void **p, size_t *cap, size_t bytes) {
  if (*cap >= bytes && *p) return TRUST_TC_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t want = std::max<size_t>(bytes, 256);
  TC_CUDA_TRY(cudaMalloc(p, want));
  *cap = want;
  return TRUST_TC_OK;
}

static int ceil_log2_size(int64_t x) {
  int l = 0;
  while (((int64_t)1 << l) < x) ++l;
  return l;
}

// Resolved launch configuration for one counting call.
struct LaunchCfg {
  int threads, blocks, chunk, warp_max, cta_max, cta_log2, warp_slots;
  size_t smem;
};

static int resolve_cfg(trust_tc_ctx *c, const trust_tc_opts &o, bool same, LaunchCfg *cfg) {
  cfg->threads = o.threads_per_block > 0 ? o.threads_per_block : 256;
  if (cfg->threads % 32 || cfg->threads < 64 || cfg->threads > 1024) return TRUST_TC_E_ARG;
  // the plain schedule is the reference's split: a warp per vertex up to out-degree 100 (USE_CTA);
  // the tuned and learned classes give a warp rows of up to 512 entries (measured on R-MAT 22 /
  // 24 / 26 with the learned schedule: 13 % / 5 % / 2 % faster than 128, since CTA-class rows pay
  // a CTA barrier per vertex; 1024 loses occupancy to 64 KiB of warp tables)
  cfg->warp_max = o.warp_max_degree > 0 ? o.warp_max_degree : (o.schedule == TRUST_TC_SCHED_PLAIN ? 100 : 512);
  if (cfg->warp_max < 32 || cfg->warp_max > 4096) return TRUST_TC_E_ARG;
  int want_cta = o.block_max_degree > 0 ? o.block_max_degree : 4096;
  if (want_cta < cfg->warp_max) return TRUST_TC_E_ARG;
  cfg->cta_log2 = std::max(ceil_log2_size(2 * (int64_t)want_cta), 6);
  const int warps = cfg->threads / 32;
  cfg->warp_slots = 1 << std::max(ceil_log2_size(2 * (int64_t)cfg->warp_max), 7);  // >= 4*32 for G32 groups
  size_t table_bytes = (size_t)4 << cfg->cta_log2;
  size_t warp_bytes = (size_t)4 * cfg->warp_slots * warps;
  cfg->smem = std::max(table_bytes, warp_bytes);
  if (cfg->smem > (size_t)c->max_smem_optin) return TRUST_TC_E_ARG;
  cfg->cta_max = 1 << (cfg->cta_log2 - 1);
  cfg->chunk = o.chunk > 0 ? o.chunk : 8;
  int per_sm = 0;
  int st = count_kernel_occupancy(same, cfg->threads, cfg->smem, &per_sm);
  if (st) return st;
  if (per_sm < 1) return TRUST_TC_E_ARG;
  cfg->blocks = o.blocks > 0 ? o.blocks : c->num_sms * per_sm;
  return TRUST_TC_OK;
}

// The learned schedule promotes a warp-class row to a CTA when its predicted cost exceeds
// 2^TC_PROMOTE_LOG2 cycles (about 32 ms at the GB300 clock: only a row that would hold one warp
// far longer than the whole count).  Measured on GB300 (learned call): with the bound at 2^22 the
// promotions cost 1-2 % (R-MAT 24 a = 0.70 172.1 against 169.6 ms without, R-MAT 26 ef32 2353
// against 2335 ms, R-MAT 20 5.66 against 5.69 ms), so only outliers are promoted.
constexpr float TC_PROMOTE_LOG2 = 26.f;

// Below this many arcs the learned schedule's scheduling pass cannot be repaid: on R-MAT scale 18
// (3.8M arcs, a 1.7 ms count) the split with the pass costs 2 % more than the tuned classes
// without it, on scale 19 (7.7M arcs) it saves 5 %.  Smaller graphs run the tuned schedule.
constexpr int64_t TC_LEARNED_MIN_ARCS = (int64_t)1 << 22;
// Nor where few arcs sit in long rows: the split pays through the probes of rows longer than
// TC_LONG_ROW (128) entries.  Measured on GB300: it paid on every R-MAT graph with a >= 0.57
// (scales 18-21; 34-67 % of arcs in such rows) and lost on a = 0.45 R-MAT and Chung-Lu graphs
// (0-6 %), where the pass alone cost 0.3-1.0 ms more than the tuned classes.
constexpr double TC_LEARNED_MIN_LONG_FRAC = 0.15;
// Small graphs with long rows (fewer than 2^21 arcs, a row of at least 64 entries) run the plain
// split, in 128-thread CTAs, under the learned schedule: packing 4 to 32 rows per warp leaves too few warp tasks to
// fill the GPU while the long rows hold their warps.  Measured on GB300 (call ms, default tuned
// classes vs plain): R-MAT 14 0.222 / 0.155, R-MAT 16 0.450 / 0.421, R-MAT 17 0.812 / 0.728, while
// from R-MAT 18 (3.8M arcs: 1.62 / 1.67) and on small Chung-Lu, Erdos-Renyi and Barabasi-Albert
// graphs (longest rows 18 to 29 entries: 0.09 / 0.20, 0.11 / 0.14, 0.09 / 0.12) the tuned classes win.
constexpr int64_t TC_SMALL_SKEWED_ARCS = (int64_t)1 << 21;
constexpr int TC_SMALL_SKEWED_MIN_ROW = 64;

// Make the cost model in use resident on the device: the caller's (opts.model) or the library's
// default.  Sets *d_model to null when neither is available (no decisions from a model).
static int load_model(trust_tc_ctx *c, const float *host_model, const float **d_model) {
  *d_model = nullptr;
  float tmp[TC_MODEL_FLOATS];
  const float *src = host_model;
  if (!src) {
    if (trust_tc_model_default(tmp) != TRUST_TC_OK) return TRUST_TC_OK;
    src = tmp;
  }
  int rc = ensure((void **)&c->d_model, &c->model_cap, sizeof(float) * TC_MODEL_FLOATS);
  if (rc) return rc;
  if (!c->model_loaded || memcmp(c->model_host, src, sizeof(float) * TC_MODEL_FLOATS) != 0) {
    memcpy(c->model_host, src, sizeof(float) * TC_MODEL_FLOATS);
    TC_CUDA_TRY(cudaMemcpy(c->d_model, src, sizeof(float) * TC_MODEL_FLOATS, cudaMemcpyHostToDevice));
    c->model_loaded = 1;
  }
  *d_model = c->d_model;
  return TRUST_TC_OK;
}

// Whether the direction split is worth its extra pass over the arcs and the in-list build:
// enough probes saved in absolute terms (a probe-heavy graph) and relatively.
static bool split_pays(unsigned long long w_all, unsigned long long w_min, int64_t m, int64_t n) {
  if (w_all == 0 || m == 0) return false;
  const double saved = (double)(w_all - w_min);
  return (double)w_min <= 0.8 * (double)w_all && saved >= 32.0 * (double)(m + n);
}

static int split_second_pass(trust_tc_ctx *c, const DevGraph3 &g, const trust_tc_opts &o, bool same,
                             int64_t max_out_degree, trust_tc_result *rb, float *t_build);

// The device-side counting call over three CSRs (A = tables, B = arcs, C = probe lists).
// `check_*` select which CSRs get an id-range check on the device.
int count_device(trust_tc_ctx *c, const DevGraph3 &g, const trust_tc_opts &o, bool check_ids,
                 trust_tc_result *r) {
  cudaStream_t st = (cudaStream_t)o.stream;
  const bool same = g.begA == g.begB && g.begB == g.begC && g.adjA == g.adjB && g.adjB == g.adjC;
  LaunchCfg cfg;
  int rc = resolve_cfg(c, o, same, &cfg);
  if (rc) return rc;
  TcControl *ctl = c->d_ctl;
  // source rows whose arcs are counted (one CSR): [row_lo, row_hi); row_hi = -1 means all rows
  const int64_t row_lo = g.row_lo, row_hi = g.row_hi > 0 ? g.row_hi : -1;
  TC_CUDA_TRY(cudaEventRecord(c->ev[0], st));
  TC_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(TcControl), st));
  ListOffsets off{};
  // one CSR: validation, class histogram and list scatter in one kernel, each class listed in a
  // fixed range of the list buffer (7 rows entries), so no offsets wait for the host
  const bool fused = same && !g.rowmap && 7 * g.rows < ((int64_t)1 << 31);
  // a small graph under the default learned schedule is listed under the plain split as well (the
  // second 7 rows entries), so the host can take it after the one readback
  const bool small_alt = fused && o.schedule == TRUST_TC_SCHED_LEARNED && o.warp_max_degree <= 0 &&
                         o.direction_split != 1 && g.min_deg == 2 && g.mA < TC_SMALL_SKEWED_ARCS &&
                         14 * g.rows < ((int64_t)1 << 31);
  if (fused) {
    rc = ensure((void **)&c->d_lists, &c->lists_cap,
                sizeof(int) * (size_t)std::max<int64_t>((small_alt ? 14 : 7) * g.rows, 1));
    if (rc) return rc;
    TC_CUDA_TRY(cudaEventRecord(c->ev[1], st));
    rc = launch_check_classify(g.begA, g.adjA, g.rows, g.mA, check_ids, g.min_deg, cfg.warp_max, cfg.cta_max,
                               o.schedule, ctl, c->d_lists, c->num_sms, st, row_lo, row_hi,
                               small_alt ? c->d_lists + 7 * g.rows : nullptr);
    if (rc) return rc;
  } else {
    // 1. validation of every distinct CSR: offsets always, ids on request
    const int64_t rowsA = g.rowmap ? g.rowsA : g.rows;
    rc = launch_check(g.begA, g.adjA, rowsA, g.mA, g.boundA, check_ids, ctl, c->num_sms, st);
    if (rc) return rc;
    if (!same) {
      rc = launch_check(g.begB, g.adjB, g.rows, g.mB, g.boundB, check_ids, ctl, c->num_sms, st);
      if (rc) return rc;
      if (g.begC != g.begA || g.adjC != g.adjA) {
        rc = launch_check(g.begC, g.adjC, g.rowsC, g.mC, g.boundC, check_ids, ctl, c->num_sms, st);
        if (rc) return rc;
      }
    }
    // 2. classification histogram
    TC_CUDA_TRY(cudaEventRecord(c->ev[1], st));
    rc = launch_classify(0, g.begA, g.begB, g.rows, g.min_deg, cfg.warp_max, cfg.cta_max, ctl, c->d_lists,
                         off, c->num_sms, st, o.schedule, g.rowmap, nullptr, row_lo, row_hi);
    if (rc) return rc;
  }
  TC_CUDA_TRY(cudaMemcpyAsync(c->h_ctl, ctl, sizeof(TcControl), cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  TcControl h = *c->h_ctl;
  if (h.status & TC_DEV_BAD_OFFSETS) return TRUST_TC_E_OFFSETS;
  if (h.status & TC_DEV_TOO_LARGE) return TRUST_TC_E_TOO_LARGE;
  if (h.status & TC_DEV_BAD_IDS) return TRUST_TC_E_IDS;
  const bool plain_small = small_alt && h.max_out_degree >= TC_SMALL_SKEWED_MIN_ROW;
  if (plain_small) {
    // the kernels read every class's size from the device control block: it must hold the plain
    // split's sizes too, or they would walk past the ends of the plain lists
    memcpy(h.class_count, h.class_count_alt, sizeof h.class_count);
    TC_CUDA_TRY(cudaMemcpyAsync(ctl->class_count, ctl->class_count_alt, sizeof ctl->class_count,
                                cudaMemcpyDeviceToDevice, st));
    cfg.warp_max = TC_PLAIN_WARP_MAX;
    // and 128-thread CTAs unless the caller chose: R-MAT 16 0.377 ms against 0.423 with 256, R-MAT
    // 17 0.686 against 0.733 (GB300); the grid is sized from the occupancy of this shape below
    if (o.threads_per_block <= 0) cfg.threads = 128;
  }
  // Learned schedule: one scheduling pass over the arcs (split plan, and with a cost model the
  // predicted cycles and class decision of every row longer than 32), then the direction split
  // decision; the decisions re-run the class histogram.
  int split = 0;
  float saving_ms = 0.f;
  const unsigned char *dec = nullptr;
  const float *pred = nullptr;
  const bool learned = o.schedule == TRUST_TC_SCHED_LEARNED && same && g.min_deg == 2 && g.rows > 0;
  // the pass is only worth running on skewed rows (short rows bound what it can change) of a
  // graph large enough to repay it (it costs about two traversals of the arcs)
  const bool consider =
      same && g.min_deg == 2 && g.rows > 0 &&
      (o.direction_split == 1 || (learned && h.max_out_degree >= 64 && g.mA >= TC_LEARNED_MIN_ARCS &&
                                  (!fused || (double)h.long_arcs >= TC_LEARNED_MIN_LONG_FRAC * (double)g.mA)));
  if (consider) {
    const float *d_model = nullptr;
    if (learned) {
      rc = load_model(c, o.model, &d_model);
      if (rc) return rc;
    }
    // (the pass also checks that rows are duplicate-free, which the split needs); with a model,
    // the class histogram under its decisions follows on the stream before the one readback
    rc = split_plan(c, g.begA, g.adjA, g.rows, g.mA, st, d_model, cfg.warp_max, cfg.cta_max, TC_PROMOTE_LOG2,
                    cfg.threads / 32, ctl, row_lo, row_hi);
    if (rc) return rc;
    if (d_model) {
      dec = c->d_dec;
      pred = c->d_pred;
      TC_CUDA_TRY(cudaMemsetAsync(ctl->class_count, 0, sizeof ctl->class_count, st));
      rc = launch_classify(0, g.begA, g.begB, g.rows, g.min_deg, cfg.warp_max, cfg.cta_max, ctl, c->d_lists, off,
                           c->num_sms, st, o.schedule, g.rowmap, dec, row_lo, row_hi);
      if (rc) return rc;
    }
    TC_CUDA_TRY(cudaMemcpyAsync(c->h_ctl, ctl, sizeof(TcControl), cudaMemcpyDeviceToHost, st));
    TC_CUDA_TRY(cudaStreamSynchronize(st));
    SchedPlan plan{};
    split_plan_read(c, &plan);
    if (plan.overflow) return TRUST_TC_E_DEVICE;
    if (d_model) memcpy(h.class_count, c->h_ctl->class_count, sizeof h.class_count);
    const bool sorted = !(c->h_ctl->status & TC_DEV_UNSORTED);
    if (o.direction_split == 0) {
      split = 0;
    } else if (o.direction_split == 1) {
      split = sorted;
    } else if (d_model) {
      // predicted saving (warp-cycles spread over the resident warps) against the cost of the
      // in-list build and second-pass setup, with a 1.5x margin
      const double warps = (double)c->num_sms * (double)std::max(cfg.blocks / std::max(c->num_sms, 1), 1) *
                           (double)(cfg.threads / 32);
      const double saved_ms = (double)plan.saved_cycles / (warps * (double)std::max(c->clock_khz, 1));
      const double cost_ms = 0.05 + 3.5e-8 * (double)g.mA;
      saving_ms = (float)saved_ms;
      split = sorted && saved_ms > 1.5 * cost_ms;
    } else {
      split = sorted && split_pays(plan.w_all, plan.w_min, g.mA, g.rows);
    }
  }
  // a tile job (three CSRs, duplicate-free tables and probe rows): the same split, decided by the
  // probe totals of its plan
  const bool consider3 = !same && g.split_ok && !g.rowmap && g.rows > 0 && g.min_deg == 1 &&
                         (o.direction_split == 1 ||
                          (o.direction_split < 0 && o.schedule == TRUST_TC_SCHED_LEARNED &&
                           h.max_out_degree >= 64 && g.mB >= TC_LEARNED_MIN_ARCS));
  if (consider3) {
    rc = tile_split_plan(c, g, st);
    if (rc) return rc;
    TC_CUDA_TRY(cudaStreamSynchronize(st));
    SchedPlan plan{};
    split_plan_read(c, &plan);
    if (plan.overflow) return TRUST_TC_E_DEVICE;
    split = o.direction_split == 1 || split_pays(plan.w_all, plan.w_min, g.mB, g.rows);
  }
  // the fused pass's lists stand unless the learned decisions re-classified the rows
  const bool lists_done = fused && !dec;
  int64_t total = 0;
  for (int k = TC_CLASS_SKIP + 1; k < TC_NUM_CLASSES; ++k) {
    off.off[k] = lists_done ? (int)((plain_small ? 7 + k - 1 : k - 1) * g.rows) : (int)total;
    total += h.class_count[k];
  }
  if (!lists_done) {
    rc = ensure((void **)&c->d_lists, &c->lists_cap, (size_t)std::max<int64_t>(total, 1) * sizeof(int));
    if (rc) return rc;
  }
  CountArgs a{};
  // huge class: hub rows in shared memory - one CTA while the table fits in 64 KiB, above that a
  // thread-block cluster with the table split over its CTAs' shared memory (up to 8 CTAs, up to
  // the opt-in limit each); rows beyond that, or all of them with hub_cluster = -1, use one
  // global spill table per participating CTA.  Measured on R-MAT 26 ef32 (16,384-slot tables):
  // one CTA 3.44 s, clusters of 2 / 4 CTAs 4.30 / 5.77 s, global tables 3.63 s.
  int hub_log2C = -1, hub_max_log2 = 0, hub_clusters = 0;
  const int64_t table_max = g.max_deg_A > 0 ? g.max_deg_A : h.max_out_degree;  // largest table row
  if (h.class_count[TC_CLASS_HUGE] > 0 && o.hub_cluster >= 0) {
    const int tlog2 = std::max(ceil_log2_size(2 * table_max), 6);
    if (o.hub_cluster > 0) {
      hub_log2C = ceil_log2_size(o.hub_cluster);
      if ((1 << hub_log2C) != o.hub_cluster || hub_log2C > 3) return TRUST_TC_E_ARG;
    } else {
      hub_log2C = std::min(std::max(tlog2 - 14, 0), 3);
    }
    // the share and a staging buffer of half its size must fit one CTA's opt-in shared memory
    const int share_cap_log2 = ceil_log2_size((int64_t)(c->max_smem_optin - 2048) * 2 / 3 / 4 + 1) - 1;
    hub_max_log2 = std::min(tlog2, share_cap_log2 + hub_log2C);
    hub_log2C = std::min(hub_log2C, hub_max_log2 - 3);  // at least 8 slots per CTA
    a.hub_max_degree = 1 << (hub_max_log2 - 1);
    hub_clusters = std::max(1, std::min(h.class_count[TC_CLASS_HUGE], (2 * c->num_sms) >> hub_log2C));
  }
  if (h.class_count[TC_CLASS_HUGE] > 0 && table_max > a.hub_max_degree) {
    a.huge_log2 = ceil_log2_size(2 * table_max);
    size_t per = (size_t)4 << a.huge_log2;
    size_t budget = (size_t)1 << 31;  // 2 GiB of spill tables at most
    int nb = (int)std::min<size_t>(std::max<size_t>(budget / per, 1), (size_t)cfg.blocks);
    nb = std::min(nb, h.class_count[TC_CLASS_HUGE]);
    a.huge_blocks = nb;
    rc = ensure((void **)&c->d_huge, &c->huge_cap, per * nb);
    if (rc) return rc;
  }
  // shared memory sized to what this graph needs: warp tables, plus a CTA table only as large as
  // the largest CTA-class row present; the rest of the SM's unified memory stays L1
  // warp tables sized to the largest row a warp can get here (>= 128 slots: 4G for G32 groups)
  const int warp_slots = 1 << std::max(ceil_log2_size(2 * std::min<int64_t>(table_max, cfg.warp_max)), 7);
  size_t smem = (size_t)4 * warp_slots * (cfg.threads / 32);
  // quotient tables for the CTA class when every key and probe id has at most 26 bits; the CTA
  // table's bytes then also hold a 512-byte overflow list (tc_count.cu, TC_Q16_OVERFLOW)
  const int key_bits = ceil_log2_size(std::max<int64_t>(std::max(g.boundA, g.boundC), 2));
  const bool q16 = key_bits <= 26;
  if (h.class_count[TC_CLASS_CTA] > 0) {
    const int64_t dcta = std::min<int64_t>(h.max_out_degree, cfg.cta_max);
    smem = std::max(smem, ((size_t)4 << std::max(ceil_log2_size(2 * dcta), 6)) + (q16 ? 512 : 0));
  }
  int blocks = cfg.blocks;
  {
    int per_sm = 0;
    rc = count_kernel_occupancy(same, cfg.threads, smem, &per_sm);
    if (rc) return rc;
    if (o.blocks <= 0) blocks = c->num_sms * std::max(per_sm, 1);
    rc = set_count_kernel_carveout(same, cfg.threads, smem, std::max(per_sm, 1));
    if (rc) return rc;
  }
  // 3. scatter the class lists
  if (!lists_done) {
    rc = launch_classify(1, g.begA, g.begB, g.rows, g.min_deg, cfg.warp_max, cfg.cta_max, ctl, c->d_lists,
                         off, c->num_sms, st, o.schedule, g.rowmap, dec, row_lo, row_hi);
    if (rc) return rc;
  }
  if (pred) {  // heaviest first inside the huge, CTA and warp queues
    rc = lpt_sort(c, c->d_lists, off.off, h.class_count, pred, st);
    if (rc) return rc;
  }
  // 4. count
  a.begA = g.begA; a.begB = g.begB; a.begC = g.begC;
  a.adjA = g.adjA; a.adjB = g.adjB; a.adjC = g.adjC;
  a.rows = g.rows;
  a.lists = c->d_lists;
  a.off = off;
  a.ctl = ctl;
  a.huge_tables = c->d_huge;
  a.warp_slots = warp_slots;
  a.chunk = cfg.chunk;
  a.split = split;
  a.rowmap = g.rowmap;
  a.test_wait_expiry = o.test_wait_expiry;
  a.key_bits = q16 ? key_bits : 0;
  a.cta_table_bytes = (int)smem;
  if (h.class_count[TC_CLASS_CTA] > 0) {
    // long-row lists: one per CTA, as long as the largest CTA-class row
    const int cap = (int)std::min<int64_t>(h.max_out_degree, cfg.cta_max);
    rc = ensure((void **)&c->d_long, &c->long_cap, sizeof(int2) * (size_t)cap * (size_t)blocks);
    if (rc) return rc;
    a.long_rows = c->d_long;
    a.long_cap = cap;
  }
  a.cycles = o.record_cycles ? (unsigned long long *)r->vertex_cycles : nullptr;
  if (o.record_cycles && !r->vertex_cycles) return TRUST_TC_E_ARG;
  if (a.cycles) TC_CUDA_TRY(cudaMemsetAsync(a.cycles, 0, sizeof(unsigned long long) * (size_t)g.rows, st));
  TC_CUDA_TRY(cudaEventRecord(c->ev[2], st));
  if (a.hub_max_degree > 0) {
    rc = launch_hub(same, a, hub_max_log2, hub_log2C, hub_clusters, st);
    if (rc) return rc;
  }
  rc = launch_count(same, a, blocks, cfg.threads, smem, st);
  if (rc) return rc;
  TC_CUDA_TRY(cudaEventRecord(c->ev[3], st));
  TC_CUDA_TRY(cudaMemcpyAsync(c->h_ctl, ctl, sizeof(TcControl), cudaMemcpyDeviceToHost, st));
  trust_tc_result rb;
  memset(&rb, 0, sizeof rb);
  float t_build = 0;
  int rb_status = 0;  // TC_DEV_* bits of the second pass
  if (split) {
    // Second pass: arcs (v,u) with d(u) > d(v), hashed on u's row, streaming the sources' rows (a
    // tile job: tables from C's rows, probe rows from A's).  It runs on the context's second stream
    // with a second context's scratch while the first pass still counts: the scheduling pass's
    // outputs it reads are complete (the host has read their totals), and it writes nothing the
    // first pass reads.  Its in-list build and setup (host round trips included) hide under the
    // first pass, and its CTAs take SMs as the first pass's tail drains.
    rc = split_second_pass(c, g, o, same, h.max_out_degree, &rb, &t_build);
    if (rc == TRUST_TC_E_DEVICE) {  // its result is filled; reported with the first pass's below
      rb_status = TC_DEV_WAIT_LIMIT;
      rc = TRUST_TC_OK;
    }
    if (rc) {
      cudaStreamSynchronize(st);
      return rc;
    }
    TC_CUDA_TRY(cudaStreamWaitEvent(st, c->ev_split[2], 0));
  }
  TC_CUDA_TRY(cudaEventRecord(c->ev[4], st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  const TcControl done = *c->h_ctl;
  float t_kernel = 0, t_count = 0, t_call = 0;
  TC_CUDA_TRY(cudaEventElapsedTime(&t_kernel, c->ev[1], c->ev[3]));
  TC_CUDA_TRY(cudaEventElapsedTime(&t_count, c->ev[2], c->ev[3]));
  TC_CUDA_TRY(cudaEventElapsedTime(&t_call, c->ev[0], c->ev[4]));
  if (split) {  // classification (counting) to the end of whichever pass ends last
    float t_end_b = 0, t_count_b = 0;
    TC_CUDA_TRY(cudaEventElapsedTime(&t_end_b, c->ev[1], c->ev_split[2]));
    TC_CUDA_TRY(cudaEventElapsedTime(&t_count_b, c->ev[2], c->ev_split[2]));
    t_kernel = std::max(t_kernel, t_end_b);
    t_count = std::max(t_count, t_count_b);
  }
  r->triangles = done.count + rb.triangles;
  r->wedges = (int64_t)done.wedges + rb.wedges;
  r->kernel_seconds = t_kernel * 1e-3;
  // the counting kernels' wall span: from the first pass's first counting launch to the end of
  // whichever pass ends last (the two passes run at the same time on two streams)
  r->count_seconds = t_count * 1e-3;
  r->call_seconds = t_call * 1e-3;
  r->max_out_degree = done.max_out_degree;
  for (int k = 0; k < TC_NUM_CLASSES; ++k) r->class_sizes[k] = h.class_count[k];
  r->direction_split = split;
  r->split_saving_ms = saving_ms;
  // a bounded wait that ran out (the kernel fell back to plain loads: the count above is exact) or
  // a full table (never expected: tables hold twice their row) is reported after the result
  if ((done.status | rb_status) & (TC_DEV_TABLE_FULL | TC_DEV_WAIT_LIMIT)) return TRUST_TC_E_DEVICE;
  return TRUST_TC_OK;
}

// The direction split's second pass (see count_device), on c->sub_stream with c->sub's scratch.
// Records ev_split[0] / [1] around the in-list build and ev_split[2] at its end.
static int split_second_pass(trust_tc_ctx *c, const DevGraph3 &g, const trust_tc_opts &o, bool same,
                             int64_t max_out_degree, trust_tc_result *rb, float *t_build) {
  int rc;
  if (!c->sub_stream) TC_CUDA_TRY(cudaStreamCreateWithFlags(&c->sub_stream, cudaStreamNonBlocking));
  if (!c->sub) {
    c->sub = new trust_tc_ctx;
    if ((rc = ctx_init(c->sub, c->device))) {
      ctx_release(c->sub);
      delete c->sub;
      c->sub = nullptr;
      return rc;
    }
  }
  cudaStream_t sb = c->sub_stream;
  {
    SplitRows sr{};
    TC_CUDA_TRY(cudaEventRecord(c->ev_split[0], sb));
    rc = same ? split_build(c, g.begA, g.adjA, g.rows, g.mA, sb, &sr)
              : split_build(c, g.begC, g.adjC, g.rowsC, g.mB, sb, &sr);
    if (rc) return rc;
    TC_CUDA_TRY(cudaEventRecord(c->ev_split[1], sb));
    DevGraph3 gb = g;
    if (!same) {
      gb.begA = g.begC; gb.adjA = g.adjC; gb.mA = g.mC; gb.boundA = g.boundC;
      gb.begC = g.begA; gb.adjC = g.adjA; gb.mC = g.mA; gb.boundC = g.boundA;
      gb.rowsC = g.rows;
    }
    gb.begB = sr.beg;
    gb.adjB = sr.adj;
    gb.mB = sr.m;
    gb.boundB = g.rows;
    gb.rowmap = sr.rowmap;
    gb.rowsA = same ? g.rows : g.rowsC;
    gb.rows = sr.rows;
    gb.min_deg = 1;
    gb.split_ok = 0;
    gb.row_lo = gb.row_hi = 0;  // work rows are in-list chunks: the range was applied when planning
    gb.max_deg_A = max_out_degree;  // tables are whole rows (of the graph, or of C), not in-list chunks
    trust_tc_opts ob = o;
    ob.schedule = TRUST_TC_SCHED_TUNED;
    ob.record_cycles = 0;
    ob.stream = sb;
    rc = count_device(c->sub, gb, ob, false, rb);
    if (rc) return rc;
    TC_CUDA_TRY(cudaEventRecord(c->ev_split[2], sb));
    TC_CUDA_TRY(cudaEventElapsedTime(t_build, c->ev_split[0], c->ev_split[1]));
  }
  return TRUST_TC_OK;
}

}  // namespace tc

using namespace tc;

// ------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------
extern "C" {

void trust_tc_opts_init(trust_tc_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof *o);
  o->device = -1;
  o->ptr_kind = TRUST_TC_HOST;
  o->schedule = TRUST_TC_SCHED_LEARNED;
  o->validate = TRUST_TC_VALIDATE_FULL;
  o->direction_split = -1;
}

const char *trust_tc_strerror(int s) {
  switch (s) {
    case TRUST_TC_OK: return "ok";
    case TRUST_TC_E_ARG: return "invalid argument";
    case TRUST_TC_E_IO: return "cannot read or write graph files";
    case TRUST_TC_E_FORMAT: return "graph file sizes are not whole records";
    case TRUST_TC_E_OFFSETS: return "begin offsets are not a valid CSR (begin[0]!=0, decreasing, or begin[n]!=m)";
    case TRUST_TC_E_IDS: return "a neighbour id is outside [0, n)";
    case TRUST_TC_E_TOO_LARGE: return "graph exceeds limits (m or n >= 2^31, or an out-degree >= 2^26)";
    case TRUST_TC_E_CUDA: return "CUDA runtime error";
    case TRUST_TC_E_NOMEM: return "out of memory";
    case TRUST_TC_E_DEVICE: return "device-side error (table overflow or bounded wait expired)";
    case TRUST_TC_E_UNSUPPORTED: return "unsupported option combination";
    case TRUST_TC_E_NO_DEVICE: return "no CUDA device available";
    default: return "unknown status";
  }
}

const char *trust_tc_last_cuda_error(void) { return g_cuda_err; }

const char *trust_tc_version(void) { return "trust-gb300 0.1 (sm_103a)"; }

size_t trust_tc_readback_bytes(void) { return 2 * sizeof(TcControl); }

uint64_t trust_tc_kernel_launches(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

int trust_tc_ctx_create(trust_tc_ctx **out, int device) {
  if (!out) return TRUST_TC_E_ARG;
  *out = nullptr;
  trust_tc_ctx *c = new (std::nothrow) trust_tc_ctx();
  if (!c) return TRUST_TC_E_NOMEM;
  int rc = ctx_init(c, device);
  if (rc) {
    ctx_release(c);
    delete c;
    return rc;
  }
  *out = c;
  return TRUST_TC_OK;
}

int trust_tc_ctx_destroy(trust_tc_ctx *c) {
  if (!c) return TRUST_TC_E_ARG;
  ctx_release(c);
  delete c;
  return TRUST_TC_OK;
}

int trust_tc_validate_csr(const int64_t *beg, const int32_t *adj, int64_t n, int64_t m,
                          int64_t *max_out_degree) {
  if (!beg || n < 0 || m < 0 || (m > 0 && !adj)) return TRUST_TC_E_ARG;
  if (n >= ((int64_t)1 << 31) || m >= ((int64_t)1 << 31)) return TRUST_TC_E_TOO_LARGE;
  if (beg[0] != 0 || beg[n] != m) return TRUST_TC_E_OFFSETS;
  int64_t dmax = 0;
  for (int64_t v = 0; v < n; ++v) {
    int64_t d = beg[v + 1] - beg[v];
    if (d < 0) return TRUST_TC_E_OFFSETS;
    if (d >= ((int64_t)1 << 26)) return TRUST_TC_E_TOO_LARGE;
    dmax = std::max(dmax, d);
  }
  for (int64_t i = 0; i < m; ++i)
    if (adj[i] < 0 || (int64_t)adj[i] >= n) return TRUST_TC_E_IDS;
  if (max_out_degree) *max_out_degree = dmax;
  return TRUST_TC_OK;
}

int trust_tc_autotune(trust_tc_ctx *ctx, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m,
                      const trust_tc_opts *base, int repeats, double time_budget_s, trust_tc_opts *best,
                      double *best_ms) {
  if (!ctx || !best || repeats < 1 || time_budget_s < 0) return TRUST_TC_E_ARG;
  trust_tc_opts o;
  if (base) o = *base; else trust_tc_opts_init(&o);
  if (o.ptr_kind != TRUST_TC_DEVICE || o.record_cycles) return TRUST_TC_E_ARG;
  // median call time of `repeats` calls under `t`; the first call's result checks the count
  uint64_t expect = 0;
  bool have = false;
  int64_t huge = 0;
  auto time_of = [&](const trust_tc_opts &t, double *ms) -> int {
    std::vector<double> v;
    for (int k = 0; k < repeats; ++k) {
      trust_tc_result r;
      memset(&r, 0, sizeof r);
      int rc = trust_tc_count_csr(ctx, beg, adj, n, m, &t, &r);
      if (rc) return rc;
      if (have && r.triangles != expect) return TRUST_TC_E_DEVICE;  // a schedule never changes the count
      expect = r.triangles;
      have = true;
      huge = r.class_sizes[TC_CLASS_HUGE];
      v.push_back(r.call_seconds * 1e3);
    }
    std::sort(v.begin(), v.end());
    *ms = v[v.size() / 2];
    return TRUST_TC_OK;
  };
  // device time spent on candidates so far; once past the budget no new candidate starts
  double spent_ms = 0;
  const double budget_ms = time_budget_s * 1e3;
  double cur = 0;
  int rc = time_of(o, &cur);
  if (rc) return rc;
  spent_ms += cur * repeats;
  // coordinate descent over the launch parameters, each from the best so far
  auto sweep = [&](int trust_tc_opts::*field, std::initializer_list<int> values) -> int {
    for (int val : values) {
      if (o.*field == val) continue;
      if (budget_ms > 0 && spent_ms >= budget_ms) break;
      trust_tc_opts t = o;
      t.*field = val;
      double ms = 0;
      int e = time_of(t, &ms);
      if (e == TRUST_TC_E_ARG) continue;  // not a valid combination (e.g. CTA bound below the warp bound)
      if (e) return e;
      spent_ms += ms * repeats;
      if (ms < cur) {
        cur = ms;
        o = t;
      }
    }
    return TRUST_TC_OK;
  };
  // the schedule first (the plain split can win on small graphs, where the longest rows bound
  // the time), then the launch shape under it
  if ((rc = sweep(&trust_tc_opts::schedule, {TRUST_TC_SCHED_LEARNED, TRUST_TC_SCHED_TUNED, TRUST_TC_SCHED_PLAIN})))
    return rc;
  if ((rc = sweep(&trust_tc_opts::threads_per_block, {128, 256, 512, 1024}))) return rc;
  if ((rc = sweep(&trust_tc_opts::warp_max_degree, {64, 128, 256}))) return rc;
  if ((rc = sweep(&trust_tc_opts::chunk, {4, 8, 16}))) return rc;
  if (huge > 0 && (rc = sweep(&trust_tc_opts::hub_cluster, {0, 1, 2, 4, -1}))) return rc;
  *best = o;
  if (best_ms) *best_ms = cur;
  return TRUST_TC_OK;
}

int trust_tc_count_csr(trust_tc_ctx *ctx, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m,
                       const trust_tc_opts *opts, trust_tc_result *r) {
  if (!beg || !r || n < 0 || m < 0 || (m > 0 && !adj)) return TRUST_TC_E_ARG;
  trust_tc_opts o;
  if (opts) o = *opts; else trust_tc_opts_init(&o);
  if (o.ptr_kind != TRUST_TC_HOST && o.ptr_kind != TRUST_TC_DEVICE) return TRUST_TC_E_ARG;
  if (o.schedule != TRUST_TC_SCHED_PLAIN && o.schedule != TRUST_TC_SCHED_LEARNED && o.schedule != TRUST_TC_SCHED_TUNED)
    return TRUST_TC_E_ARG;
  if (n >= ((int64_t)1 << 31) || m >= ((int64_t)1 << 31)) return TRUST_TC_E_TOO_LARGE;
  if (o.row_begin < 0 || o.row_end < 0 || o.row_end > n || (o.row_end > 0 && o.row_begin > o.row_end) ||
      (o.row_end == 0 && o.row_begin > n))
    return TRUST_TC_E_ARG;
  uint64_t *cycles = r->vertex_cycles;
  memset(r, 0, sizeof *r);
  r->vertex_cycles = cycles;
  r->vertices = n;
  r->edges = m;
  int rc;
  trust_tc_ctx tmp;
  trust_tc_ctx *c = ctx;
  if (!c) {
    rc = ctx_init(&tmp, o.device);
    if (rc) { ctx_release(&tmp); return rc; }
    c = &tmp;
  } else if (o.device >= 0 && o.device != c->device) {
    return TRUST_TC_E_ARG;
  }
  if ((rc = cuda_status(cudaSetDevice(c->device)))) { if (c == &tmp) ctx_release(&tmp); return rc; }
  DevGraph3 g{};
  bool check_ids = false;
  trust_tc_ctx::Staged *slot = nullptr;
  if (o.ptr_kind == TRUST_TC_HOST) {
    cudaStream_t st = (cudaStream_t)o.stream;
    // a copy staged ahead by trust_tc_stage_csr for these host buffers: the oldest one
    for (auto &sl : c->staged)
      if (sl.waiting && sl.h_beg == beg && sl.h_adj == adj && sl.n == n && sl.m == m && (!slot || sl.seq < slot->seq))
        slot = &sl;
    if (slot) {
      rc = cuda_status(cudaStreamWaitEvent(st, slot->ready, 0));
      g.begA = g.begB = g.begC = slot->d_beg;
      g.adjA = g.adjB = g.adjC = slot->d_adj;
    } else {
      rc = ensure((void **)&c->d_beg, &c->beg_cap, sizeof(int64_t) * (size_t)(n + 1));
      if (!rc) rc = ensure((void **)&c->d_adj, &c->adj_cap, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1));
      if (!rc) rc = cuda_status(cudaMemcpyAsync(c->d_beg, beg, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice, st));
      if (!rc && m) rc = cuda_status(cudaMemcpyAsync(c->d_adj, adj, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, st));
      g.begA = g.begB = g.begC = c->d_beg;
      g.adjA = g.adjB = g.adjC = c->d_adj;
    }
    check_ids = true;  // host input is checked on the device after the copy, never skipped
  } else {
    g.begA = g.begB = g.begC = beg;
    g.adjA = g.adjB = g.adjC = adj;
    check_ids = o.validate >= TRUST_TC_VALIDATE_FULL;
  }
  if (!rc) {
    g.rows = g.rowsC = n;
    g.mA = g.mB = g.mC = m;
    g.boundA = g.boundB = g.boundC = n;
    g.min_deg = 2;
    g.row_lo = o.row_begin;
    g.row_hi = o.row_end > 0 ? o.row_end : n;
    rc = count_device(c, g, o, check_ids, r);
  }
  if (slot) {  // count_device has synchronised (or failed): the slot is free for the next stage
    if (rc) cudaStreamSynchronize((cudaStream_t)o.stream);
    slot->waiting = 0;
  }
  r->vertices = n;
  r->edges = m;
  if (c == &tmp) ctx_release(&tmp);
  return rc;
}

int trust_tc_stage_csr(trust_tc_ctx *ctx, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m) {
  if (!ctx || !beg || n < 0 || m < 0 || (m > 0 && !adj)) return TRUST_TC_E_ARG;
  if (n >= ((int64_t)1 << 31) || m >= ((int64_t)1 << 31)) return TRUST_TC_E_TOO_LARGE;
  trust_tc_ctx::Staged *sl = nullptr;
  for (auto &x : ctx->staged)
    if (!x.waiting) { sl = &x; break; }
  if (!sl) return TRUST_TC_E_ARG;  // two staged inputs are already waiting for their counts
  int rc = cuda_status(cudaSetDevice(ctx->device));
  if (rc) return rc;
  if ((rc = ensure((void **)&sl->d_beg, &sl->beg_cap, sizeof(int64_t) * (size_t)(n + 1)))) return rc;
  if ((rc = ensure((void **)&sl->d_adj, &sl->adj_cap, sizeof(int32_t) * (size_t)std::max<int64_t>(m, 1)))) return rc;
  TC_CUDA_TRY(cudaMemcpyAsync(sl->d_beg, beg, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice,
                              ctx->copy_stream));
  if (m)
    TC_CUDA_TRY(cudaMemcpyAsync(sl->d_adj, adj, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, ctx->copy_stream));
  TC_CUDA_TRY(cudaEventRecord(sl->ready, ctx->copy_stream));
  sl->h_beg = beg;
  sl->h_adj = adj;
  sl->n = n;
  sl->m = m;
  sl->seq = ++ctx->stage_seq;
  sl->waiting = 1;
  return TRUST_TC_OK;
}

void trust_tc_free_host(void *p) { free(p); }

static int64_t file_bytes(const std::string &path) {
  struct stat st;
  if (stat(path.c_str(), &st) != 0) return -1;
  return (int64_t)st.st_size;
}

static int read_all(const std::string &path, void *dst, size_t bytes) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return TRUST_TC_E_IO;
  size_t got = bytes ? fread(dst, 1, bytes, f) : 0;
  fclose(f);
  return got == bytes ? TRUST_TC_OK : TRUST_TC_E_IO;
}

int trust_tc_load_folder(const char *folder, int64_t **beg, int32_t **adj, int64_t *n, int64_t *m) {
  if (!folder || !beg || !adj || !n || !m) return TRUST_TC_E_ARG;
  *beg = nullptr;
  *adj = nullptr;
  std::string fb = std::string(folder) + "/begin.bin", fa = std::string(folder) + "/adjacent.bin";
  int64_t bb = file_bytes(fb), ab = file_bytes(fa);
  if (bb < 0 || ab < 0) return TRUST_TC_E_IO;
  if (bb < 8 || bb % 8 || ab % 4) return TRUST_TC_E_FORMAT;
  int64_t nn = bb / 8 - 1, mm = ab / 4;
  if (nn >= ((int64_t)1 << 31) || mm >= ((int64_t)1 << 31)) return TRUST_TC_E_TOO_LARGE;
  int64_t *b = (int64_t *)malloc((size_t)bb);
  int32_t *a = (int32_t *)malloc((size_t)std::max<int64_t>(ab, 4));
  if (!b || !a) { free(b); free(a); return TRUST_TC_E_NOMEM; }
  int rc = read_all(fb, b, (size_t)bb);
  if (!rc) rc = read_all(fa, a, (size_t)ab);
  if (rc) { free(b); free(a); return rc; }
  *beg = b;
  *adj = a;
  *n = nn;
  *m = mm;
  return TRUST_TC_OK;
}

int trust_tc_save_folder(const char *folder, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m) {
  if (!folder || !beg || n < 0 || m < 0 || (m && !adj)) return TRUST_TC_E_ARG;
  std::string fb = std::string(folder) + "/begin.bin", fa = std::string(folder) + "/adjacent.bin";
  FILE *f = fopen(fb.c_str(), "wb");
  if (!f) return TRUST_TC_E_IO;
  bool ok = fwrite(beg, sizeof(int64_t), (size_t)(n + 1), f) == (size_t)(n + 1);
  ok &= fclose(f) == 0;
  f = fopen(fa.c_str(), "wb");
  if (!f) return TRUST_TC_E_IO;
  if (m) ok &= fwrite(adj, sizeof(int32_t), (size_t)m, f) == (size_t)m;
  ok &= fclose(f) == 0;
  return ok ? TRUST_TC_OK : TRUST_TC_E_IO;
}

int trust_tc_vertex_features(trust_tc_ctx *ctx, const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                             float *d_features) {
  if (!ctx || !d_begin || !d_features || n < 0 || m < 0 || (m && !d_adj)) return TRUST_TC_E_ARG;
  TC_CUDA_TRY(cudaSetDevice(ctx->device));
  trust_tc_opts o;
  trust_tc_opts_init(&o);
  o.ptr_kind = TRUST_TC_DEVICE;
  LaunchCfg cfg;
  int rc = resolve_cfg(ctx, o, true, &cfg);
  if (rc) return rc;
  // the CSR must be valid before it is walked
  TC_CUDA_TRY(cudaMemset(ctx->d_ctl, 0, sizeof(TcControl)));
  rc = launch_check(d_begin, d_adj, n, m, n, 1, ctx->d_ctl, ctx->num_sms, 0);
  if (rc) return rc;
  TC_CUDA_TRY(cudaMemcpy(ctx->h_ctl, ctx->d_ctl, sizeof(TcControl), cudaMemcpyDeviceToHost));
  if (ctx->h_ctl->status & TC_DEV_BAD_OFFSETS) return TRUST_TC_E_OFFSETS;
  if (ctx->h_ctl->status & TC_DEV_TOO_LARGE) return TRUST_TC_E_TOO_LARGE;
  if (ctx->h_ctl->status & TC_DEV_BAD_IDS) return TRUST_TC_E_IDS;
  rc = vertex_features(ctx, d_begin, d_adj, n, cfg.warp_max, cfg.cta_max, d_features, 0);
  if (rc) return rc;
  TC_CUDA_TRY(cudaDeviceSynchronize());
  return TRUST_TC_OK;
}

int trust_tc_count_folder(const char *folder, const trust_tc_opts *opts, trust_tc_result *r) {
  if (!folder || !r) return TRUST_TC_E_ARG;
  int64_t *beg = nullptr, n = 0, m = 0;
  int32_t *adj = nullptr;
  int rc = trust_tc_load_folder(folder, &beg, &adj, &n, &m);
  if (rc) return rc;
  trust_tc_opts o;
  if (opts) o = *opts; else trust_tc_opts_init(&o);
  o.ptr_kind = TRUST_TC_HOST;
  rc = trust_tc_count_csr(nullptr, beg, adj, n, m, &o, r);
  free(beg);
  free(adj);
  return rc;
}

}  // extern "C"

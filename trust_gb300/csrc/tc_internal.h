// tc_internal.h — library-internal host structures shared by the translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_common.cuh"

// Device scratch reused across calls (work queues, class lists, spill tables, staging copies of
// host input).  Replaces the per-call cudaMalloc/cudaFree of Without-graph-partition/TC.cu:647-711.
struct trust_tc_ctx {
  int device = -1;
  int num_sms = 0;
  int max_smem_optin = 0;
  TcControl *d_ctl = nullptr;
  TcControl *h_ctl = nullptr;  // pinned
  int *d_lists = nullptr;
  size_t lists_cap = 0;
  int *d_huge = nullptr;
  size_t huge_cap = 0;
  int2 *d_long = nullptr;  // per-CTA deferred long-row lists of the CTA class
  size_t long_cap = 0;
  unsigned *d_split_cnt = nullptr;  // direction split: in-degree counts / scatter cursors
  size_t split_cnt_cap = 0;
  unsigned char *d_dec = nullptr;  // learned schedule: class decision of every row longer than 32
  size_t dec_cap = 0;
  float *d_pred = nullptr;  // learned schedule: predicted log2 cycles of those rows
  size_t pred_cap = 0;
  float *d_model = nullptr;  // the cost model in use (TC_MODEL_FLOATS)
  size_t model_cap = 0;
  float model_host[1400];    // host copy of what d_model holds (reload only on change)
  int model_loaded = 0;
  unsigned long long *d_sort = nullptr;  // heaviest-first sort: histogram, cursors, sorted copy
  size_t sort_cap = 0;
  int clock_khz = 0;
  unsigned long long *d_split_wsum = nullptr;  // per target: probes the second pass makes against it
  size_t split_wsum_cap = 0;
  unsigned long long *d_split_plans = nullptr;  // probe totals of both plans, saving, long rows
  size_t split_plans_cap = 0;
  unsigned long long *h_plans = nullptr;        // pinned host copy of d_split_plans
  int2 *d_split_pairs = nullptr;  // scheduling pass: the arcs the split would move, (target, source)
  size_t split_pairs_cap = 0;
  int *d_sched_long = nullptr;  // scheduling pass: the rows it walks a warp each
  size_t sched_long_cap = 0;
  int64_t *d_split_beg = nullptr;  // in-list offsets of the arcs sent to the second pass
  size_t split_beg_cap = 0;
  int64_t *d_split_cbase = nullptr;  // first chunk of every target
  size_t split_cbase_cap = 0;
  int64_t *d_split_cbeg = nullptr;  // chunk offsets (the second pass's work rows)
  size_t split_cbeg_cap = 0;
  int *d_split_rowmap = nullptr;  // table row of every chunk
  size_t split_rowmap_cap = 0;
  int32_t *d_split_adj = nullptr;
  size_t split_adj_cap = 0;
  int64_t *d_beg = nullptr;
  size_t beg_cap = 0;
  int32_t *d_adj = nullptr;
  size_t adj_cap = 0;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_split[3] = {nullptr, nullptr, nullptr};
  // the direction split's second pass runs on its own stream with its own scratch (a context of its
  // own, made on first use) while the first pass still counts
  trust_tc_ctx *sub = nullptr;
  cudaStream_t sub_stream = nullptr;
  // host CSRs staged ahead of their count (trust_tc_stage_csr): copied on copy_stream into one of
  // two slots, consumed oldest-first by the count call given the same host pointers and sizes
  struct Staged {
    int64_t *d_beg = nullptr;
    size_t beg_cap = 0;
    int32_t *d_adj = nullptr;
    size_t adj_cap = 0;
    const int64_t *h_beg = nullptr;
    const int32_t *h_adj = nullptr;
    int64_t n = 0, m = 0;
    int waiting = 0;       // staged and not yet counted
    uint64_t seq = 0;      // staging order
    cudaEvent_t ready = nullptr;
  } staged[2];
  uint64_t stage_seq = 0;
  cudaStream_t copy_stream = nullptr;
};

namespace tc {

// Three CSRs on the device: A rows are hashed, B rows give the arcs (v,u), C rows are probed.
struct DevGraph3 {
  const int64_t *begA, *begB, *begC;
  const int32_t *adjA, *adjB, *adjC;
  const int *rowmap;          // table row (A) of every work row (B); null = the same index
  int64_t rowsA;              // rows of A when a row map is given (else = rows)
  int64_t rows;               // rows of A and B
  int64_t rowsC;              // rows of C
  int64_t mA, mB, mC;         // entries of each
  int64_t boundA, boundB, boundC;  // exclusive id bound per CSR (B's ids index rows of C)
  int min_deg;                // rows with fewer entries in A or B are skipped
  int64_t max_deg_A;          // largest row of A when known (0: the validation pass's maximum)
  int split_ok;               // three distinct CSRs whose A and C rows are duplicate-free: the
                              // direction split may count an arc from C's side
  int64_t row_lo, row_hi;     // one CSR: only arcs of source rows in [row_lo, row_hi) are counted
                              // (row_hi = 0: all rows)
};

int ctx_init(trust_tc_ctx *c, int device);
void ctx_release(trust_tc_ctx *c);
int ensure(void **p, size_t *cap, size_t bytes);
int count_device(trust_tc_ctx *c, const DevGraph3 &g, const trust_tc_opts &o, bool check_ids,
                 trust_tc_result *r);
int scan_exclusive_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t st, int64_t *total);
// The n x n hash partition of a device CSR into p*p tiles (tile i*p+j) in pinned host memory
// (free each beg / adj with cudaFreeHost); p <= 32.
struct PinnedTile {
  int64_t *beg;
  int32_t *adj;
  int64_t rows, m;
};
int partition_device_to_host(const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, int p, PinnedTile *tiles);
constexpr int TC_PLAN_WORDS = 8;  // words of the scheduling pass's totals
struct SchedPlan {
  unsigned long long w_all, w_min;  // probes without / with the direction split
  float saved_cycles;               // model: predicted cycles the split saves on rows > 32
  int64_t long_rows;                // rows longer than 32 entries
  int64_t moved_arcs;               // pair slots the pass used (moved arcs and holes)
  bool overflow;                    // the pair arrays ran out (never expected): no split
};
// Only source rows in [row_lo, row_hi) are walked (their arcs planned and moved).
int split_plan(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, cudaStream_t st,
               const float *d_model, int warp_max, int cta_max, float promote_log2, int cta_warps, TcControl *ctl,
               int64_t row_lo, int64_t row_hi);
// after the stream has synchronised
void split_plan_read(const trust_tc_ctx *c, SchedPlan *plan);
int radix_sort_u64(unsigned long long *keys, unsigned long long *tmp, int64_t n, const int *shifts, int nshifts,
                   cudaStream_t st);
// heaviest first: reorder the list of each of the given classes by predicted cycles, descending
int lpt_sort(trust_tc_ctx *c, int *lists, const int *off, const int *counts, const float *pred, cudaStream_t st);
int vertex_features(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int warp_max,
                    int cta_max, float *d_features, cudaStream_t st);
// work rows of the second pass: at least max(TC_SPLIT_WORK_PER_ENTRY * d(u), TC_SPLIT_MIN_WORK)
// probes each, so the table rebuild stays a small fraction of a row's work
constexpr int TC_SPLIT_WORK_PER_ENTRY = 256;
constexpr int TC_SPLIT_MIN_WORK = 131072;
struct SplitRows {
  const int64_t *beg;
  const int32_t *adj;
  const int *rowmap;
  int64_t rows, m;
};
int split_build(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m, cudaStream_t st,
                SplitRows *out);
// The split plan of a job over three CSRs (tile jobs): probe totals and the arcs of B to move,
// read back like split_plan's.
int tile_split_plan(trust_tc_ctx *c, const DevGraph3 &g, cudaStream_t st);
// Whether every row of a CSR is strictly increasing (so duplicate-free); synchronous.
int rows_increasing(trust_tc_ctx *c, const int64_t *beg, const int32_t *adj, int64_t rows, cudaStream_t st,
                    bool *out);

}  // namespace tc

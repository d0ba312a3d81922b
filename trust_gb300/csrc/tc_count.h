// tc_count.h — host-visible interface of the counting kernels (internal to the library).
#pragma once
#include "tc_common.cuh"

namespace tc {

// The plain split's warp bound: the reference's USE_CTA (Without-graph-partition/TC.cu:19).
constexpr int TC_PLAIN_WARP_MAX = 100;

struct ListOffsets {
  int off[TC_NUM_CLASSES];  // start of each class list inside the concatenated list buffer
};

// Arguments of the persistent counting kernel.  A = rows hashed into tables, B = rows whose arcs
// (v,u) are walked, C = rows probed (N+(u)).  For a whole graph A = B = C; for an (i,j,k) tile
// job of the partitioned path A = part(i,j), B = part(i,k), C = part(k,j)
// (With-graph-partition/TC.cu:992-994).
struct CountArgs {
  const int64_t *begA, *begB, *begC;
  const int32_t *adjA, *adjB, *adjC;
  int64_t rows;
  const int *lists;
  ListOffsets off;
  TcControl *ctl;
  int *huge_tables;   // global tables for the huge class: huge_blocks regions of 2^huge_log2 ints
  int huge_log2;
  int huge_blocks;
  int warp_slots;     // shared-memory ints per warp in the warp phase
  int chunk;          // items per queue claim (per group) in the warp phase
  unsigned long long *cycles;  // optional: per-row clock64 cycles (rows * 1 entries) or null
  int split;          // 1: skip arcs (v,u) whose probe row C[u] is longer than the table row A[v];
                      // a second pass counts them from u's side
  const int *rowmap;  // optional: table row (A) of each work row (B); null = the same index
  int2 *long_rows;    // optional: per-CTA lists of deferred long neighbour rows (row start, length)
  int long_cap;       // entries per CTA in long_rows (>= the largest CTA-class out-degree)
  // batches (the disjoint union of many graphs): graph of every row, per-graph counts (both null
  // otherwise), and list offsets read from ctl->class_off on the device instead of `off`
  const int *graph_of;
  unsigned long long *graph_counts;
  int dev_off;
  // huge rows up to this out-degree are counted by hub_kernel in shared memory (0: none)
  int hub_max_degree;
  // failure-detection test: hub_kernel arms its copy barrier without issuing the copy and waits
  // a few thousand cycles, so the bounded wait runs out with nothing in flight
  int test_wait_expiry;
  // CTA-class tables: every key (entry of A) and probe (entry of C) is below 2^key_bits (0: no
  // quotient tables), and the CTA table may use cta_table_bytes of dynamic shared memory
  int key_bits;
  int cta_table_bytes;
};

int launch_check(const int64_t *beg, const int32_t *adj, int64_t rows, int64_t m, int64_t id_bound,
                 int check_ids, TcControl *ctl, int num_sms, cudaStream_t st);
// One CSR: validation + class histogram + scatter in one kernel; class c (>= 1) is listed at
// lists[(c-1) rows ...] and class_count[c] is its size.  lists holds 7 rows entries.
// Rows outside [row_lo, row_hi) (row_hi < 0: all rows) are validated but classed as skipped.
// alt_lists (7 rows entries, or null): every row also classed under the plain split there.
int launch_check_classify(const int64_t *beg, const int32_t *adj, int64_t rows, int64_t m, int check_ids,
                          int min_deg, int warp_max, int cta_max, int schedule, TcControl *ctl, int *lists,
                          int num_sms, cudaStream_t st, int64_t row_lo = 0, int64_t row_hi = -1,
                          int *alt_lists = nullptr);
int launch_classify(int pass, const int64_t *begA, const int64_t *begB, int64_t rows, int min_deg,
                    int warp_max, int cta_max, TcControl *ctl, int *lists, const ListOffsets &off,
                    int num_sms, cudaStream_t st, int schedule = TRUST_TC_SCHED_TUNED,
                    const int *rowmap = nullptr, const unsigned char *dec = nullptr, int64_t row_lo = 0,
                    int64_t row_hi = -1);
// batches: graphs fall into TC_BATCH_CLASSES size classes, each with its own degree thresholds
constexpr int TC_BATCH_CLASSES = 4;
struct BatchThresholds {
  int warp_max[TC_BATCH_CLASSES];
  int cta_max[TC_BATCH_CLASSES];
};
int launch_batch_classify(int pass, const int64_t *beg, int64_t rows, const int *graph_of,
                          const unsigned char *graph_sc, const BatchThresholds &th, TcControl *ctl, int *lists,
                          int num_sms, cudaStream_t st);
int launch_batch_offsets(TcControl *ctl, int nsc, cudaStream_t st);
// Hub rows (huge class, out-degree <= a.hub_max_degree) on clusters of 2^log2C CTAs of 512
// threads; tables up to 2^max_log2 slots, 2^(max_log2 - log2C) per CTA in shared memory.
int launch_hub(bool same, const CountArgs &a, int max_log2, int log2C, int clusters, cudaStream_t st);
int count_kernel_occupancy(bool same, int threads, size_t smem_bytes, int *blocks_per_sm);
// Shared-memory carveout hint: just enough for `per_sm` resident CTAs of `smem_bytes` each.
int set_count_kernel_carveout(bool same, int threads, size_t smem_bytes, int per_sm);
int launch_count(bool same, const CountArgs &a, int blocks, int threads, size_t smem_bytes,
                 cudaStream_t st);

}  // namespace tc

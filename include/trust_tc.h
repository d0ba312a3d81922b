/*
 * trust_tc.h — C ABI of the GB300 (sm_103a) vertex-centric hash triangle counter.
 *
 * Drop-in boundary for TRUST's counting path.  The reference exposes one C++ operator,
 *   struct arguments Triangle_count(int rank, char name[100], struct arguments args,
 *                                   int total_process, int n_threads, int n_blocks, int chunk_size)
 * (Without-graph-partition/TC.cuh:10, implemented at Without-graph-partition/TC.cu:602-731), and a
 * partitioned variant with an extra `partition_num` argument (With-graph-partition/TC.cuh:10,
 * With-graph-partition/TC.cu:976-1157).  That operator loads `begin.bin` (int64 offsets) and
 * `adjacent.bin` (int32 neighbours) from a folder, runs the `dynamic_assign` kernel and returns
 * the u64 count.  Every entry point below is plain C: pointers, sizes and status codes.  No
 * entry point calls exit(); errors come back as TRUST_TC_E_* codes (the reference prints and
 * exits on any CUDA error, Without-graph-partition/herror.h:1-8).
 *
 * Counted quantity (identical to dynamic_assign on inputs where that kernel is exact):
 *   count = sum over vertices v with out-degree d(v) >= 2,
 *           sum over arcs (v,u) in row v (with multiplicity),
 *           sum over arcs (u,w) in row u (with multiplicity),  [w is an element of row v]
 * On an oriented simple graph this is the number of triangles.  Rows may be unsorted.
 */
#ifndef TRUST_TC_H
#define TRUST_TC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
enum {
  TRUST_TC_OK = 0,
  TRUST_TC_E_ARG = 1,          /* null pointer, negative size, bad option value            */
  TRUST_TC_E_IO = 2,           /* folder / file missing or unreadable                      */
  TRUST_TC_E_FORMAT = 3,       /* file sizes not a whole number of records, n < 0          */
  TRUST_TC_E_OFFSETS = 4,      /* begin[0] != 0, begin not monotone, begin[n] != m         */
  TRUST_TC_E_IDS = 5,          /* a neighbour id outside [0, n)                            */
  TRUST_TC_E_TOO_LARGE = 6,    /* m >= 2^31, n >= 2^31 or an out-degree >= 2^26            */
  TRUST_TC_E_CUDA = 7,         /* CUDA runtime error (text in trust_tc_last_cuda_error)    */
  TRUST_TC_E_NOMEM = 8,        /* host or device allocation failed                         */
  TRUST_TC_E_DEVICE = 9,       /* device-side error word set (bounded wait ran out, ...)   */
  TRUST_TC_E_UNSUPPORTED = 10, /* option combination not supported                         */
  TRUST_TC_E_NO_DEVICE = 11    /* no CUDA device visible                                   */
};

/* where the caller's CSR arrays live */
enum { TRUST_TC_HOST = 0, TRUST_TC_DEVICE = 1 };

/* work schedule; only the schedule changes, never the integer arithmetic */
enum {
  TRUST_TC_SCHED_PLAIN = 0,   /* the reference's split: one warp per vertex for out-degree 2..100,
                                 one CTA above (USE_WARP / USE_CTA, Without-graph-partition/TC.cu:19-20) */
  TRUST_TC_SCHED_LEARNED = 1, /* (default) TUNED classes; on graphs of at least 2^22 arcs with at least
                                 15 % of them in rows longer than 128 entries (skewed rows) a
                                 scheduling pass runs a per-vertex cost model that promotes
                                 heavy vertices to CTA granularity, orders the warp, CTA and huge
                                 queues by predicted cost and decides the direction split from its
                                 predicted saving                                                    */
  TRUST_TC_SCHED_TUNED = 2    /* sub-warp degree classes (4, 8, 16, 32 lanes), warp, CTA             */
};

/* validation level for device-resident input (host input is always fully validated) */
enum { TRUST_TC_VALIDATE_NONE = 0, TRUST_TC_VALIDATE_OFFSETS = 1, TRUST_TC_VALIDATE_FULL = 2 };

typedef struct trust_tc_opts {
  int device;            /* CUDA ordinal; -1 = current device                                   */
  int threads_per_block; /* reference argv[3]; multiple of 32 in [64,1024]; 0 = library default */
  int blocks;            /* reference argv[4]; 0 = persistent (SM count x resident blocks)      */
  int chunk;             /* reference argv[5]; vertices per work-queue claim; 0 = default       */
  int ptr_kind;          /* TRUST_TC_HOST or TRUST_TC_DEVICE                                     */
  int schedule;          /* TRUST_TC_SCHED_*                                                     */
  int validate;          /* TRUST_TC_VALIDATE_* (device input); default FULL                     */
  int warp_max_degree;   /* out-degree above which a vertex gets a whole CTA; 0 = default (512;
                            100 under TRUST_TC_SCHED_PLAIN)                                   */
  int block_max_degree;  /* out-degree above which a vertex gets a cluster table; 0 = default   */
  int record_cycles;     /* 1: write per-vertex clock64 cycles into result->vertex_cycles       */
  void *stream;          /* cudaStream_t; NULL = legacy default stream                          */
  const float *model;    /* learned schedule: packed MLP weights (trust_tc_model_size floats)   */
  int direction_split;   /* charge arcs with d(u) > d(v) to u's side (hash N+(u), stream N+(v)):
                            -1 = the learned schedule decides, 0 = never, 1 = always; applied only
                            when every row is strictly increasing (duplicate-free).  In the tile
                            loop a job (i,j,k) charges arc (v,u) to u's side when its probe row
                            in tile (k,j) is longer than v's table row in tile (i,j)          */
  int hub_cluster;       /* rows above the CTA table (out-degree > 4096): 0 = in shared memory,
                            one CTA while the table fits in 64 KiB, else a thread-block cluster
                            with the table split over its CTAs (distributed shared memory);
                            1/2/4/8 = that cluster size; -1 = per-CTA global tables          */
  int64_t row_begin;     /* trust_tc_count_csr / _folder: count only the arcs (v,u) whose source
                            row v lies in [row_begin, row_end); row_end = 0 means n (the whole
                            graph).  Every row is still validated and still serves as a probe
                            row, and the schedule (classes, direction split) is decided the same
                            way, so slices of a graph sum to its count.  Other entry points
                            return TRUST_TC_E_UNSUPPORTED for a range.  No counterpart in the
                            reference, whose ranks split the vertex chunks instead
                            (Without-graph-partition/TC.cu:259, :433).                        */
  int64_t row_end;
  int test_wait_expiry;  /* test only (failure detection): 1 = the hub kernel arms its copy
                            barrier without issuing the copy and waits a few thousand cycles, so
                            the bounded wait runs out with nothing in flight; the kernel then
                            reads the rows with plain loads and the call returns
                            TRUST_TC_E_DEVICE with an exact count in the result.  0 in use.     */
} trust_tc_opts;

typedef struct trust_tc_result {
  uint64_t triangles;       /* the count                                                     */
  double kernel_seconds;    /* CUDA-event time of classification + counting (validation too in
                               a single-graph call, where it runs fused with classification) */
  double count_seconds;     /* CUDA-event time of the counting kernels alone (with the direction
                               split: from the first counting launch to the end of whichever of
                               the two concurrent passes ends last)                          */
  double call_seconds;      /* CUDA-event time of the whole device-side call                 */
  int64_t vertices;         /* n                                                            */
  int64_t edges;            /* m (oriented arcs = undirected edges)                         */
  int64_t max_out_degree;
  int64_t wedges;           /* sum over arcs (v,u) with d(v)>=2 of d(u): the probe count     */
  int64_t class_sizes[8];   /* vertices per schedule class (skip, g4, g8, g16, g32, warp, cta, cluster) */
  uint64_t *vertex_cycles;  /* caller-provided device array of n entries, or NULL            */
  int32_t direction_split;  /* 1 when the second (reverse-direction) pass ran (tile loop: the
                               number of jobs that ran it)                                  */
  float split_saving_ms;    /* learned schedule: predicted saving of that pass, ms (else 0)  */
} trust_tc_result;

typedef struct trust_tc_ctx trust_tc_ctx;

/* default option values */
void trust_tc_opts_init(trust_tc_opts *opts);

/* text for a status code (static storage) */
const char *trust_tc_strerror(int status);
/* text of the last CUDA error seen by this thread, or "" */
const char *trust_tc_last_cuda_error(void);
/* library version string */
const char *trust_tc_version(void);
/* bytes read back from the device per counting call (status words and the count) */
size_t trust_tc_readback_bytes(void);
/* kernels this library has launched since it was loaded (all threads and contexts) */
uint64_t trust_tc_kernel_launches(void);

/* A context owns device scratch (work queues, class lists, spill tables, staging copies of
 * host input) and reuses it across calls.  Not thread-safe; separate contexts are independent.
 * Replaces the per-call cudaMalloc/cudaFree of Without-graph-partition/TC.cu:655-711. */
int trust_tc_ctx_create(trust_tc_ctx **ctx, int device);
int trust_tc_ctx_destroy(trust_tc_ctx *ctx);

/* Host-side CSR check (Without-graph-partition/graph.hpp:18-67 performs none):
 * begin[0]==0, non-decreasing, begin[n]==m, ids in [0,n), m < 2^31, out-degree < 2^26.
 * On success writes the maximum out-degree to *max_out_degree (may be NULL). */
int trust_tc_validate_csr(const int64_t *begin, const int32_t *adj, int64_t n, int64_t m,
                          int64_t *max_out_degree);

/* Count over a CSR.  Replaces dynamic_assign + its launch (Without-graph-partition/TC.cu:230-600,
 * :666-696).  Arrays are borrowed; with ptr_kind HOST they are copied to ctx-owned device
 * memory inside the call.  ctx may be NULL (a temporary context is used).  On TRUST_TC_E_DEVICE
 * the result is filled as well: after an expired bounded wait the kernel re-read its rows with
 * plain loads, so the count is exact; after a table overflow (never expected) it is not. */
int trust_tc_count_csr(trust_tc_ctx *ctx, const int64_t *begin, const int32_t *adj, int64_t n,
                       int64_t m, const trust_tc_opts *opts, trust_tc_result *result);

/* Start copying a host CSR to the device on the context's own copy stream and return at once
 * (no counterpart in the reference, whose host operator copies and counts in one blocking call,
 * Without-graph-partition/TC.cu:640-696).  The next trust_tc_count_csr on this context with
 * ptr_kind HOST and the same begin/adj pointers and n, m counts the staged copy (oldest first)
 * instead of copying again, so a caller counting a stream of graphs overlaps the copy of the
 * next one with the count of the current one.  Two staged inputs may wait at a time
 * (TRUST_TC_E_ARG beyond that).  The host arrays must stay unchanged until the count that
 * consumes them returns; with pinned memory the copy is asynchronous. */
int trust_tc_stage_csr(trust_tc_ctx *ctx, const int64_t *begin, const int32_t *adj, int64_t n, int64_t m);

/* Count over a device-resident CSR without allocating anything.  No counterpart in the
 * reference: it is for callers that may not allocate GPU memory while they count (memory owned
 * by their own pool under a fixed budget, or where cudaMalloc's implicit synchronisation would
 * stall other work).  Scratch comes from one 16 MiB array in the library's device image, held by
 * every GPU that loads the library until exit.  Limits: n <= 4,194,240 rows and every out-degree
 * within the CTA table (default 4096); larger inputs return TRUST_TC_E_TOO_LARGE.  opts->ptr_kind
 * must be TRUST_TC_DEVICE and opts->record_cycles 0 (else TRUST_TC_E_UNSUPPORTED); timing fields
 * of the result stay 0.  The first call on a device looks up the array's address and keeps it for
 * the life of the process (not valid after cudaDeviceReset); make that first call before any
 * stream capture.  Every call synchronises its stream twice and returns with the caller's current
 * device unchanged.  Calls that overlap on the GPU race on the shared array and must be
 * serialised by the caller. */
int trust_tc_count_csr_noalloc(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                               const trust_tc_opts *opts, trust_tc_result *result);

/* Load `<folder>/begin.bin` and `<folder>/adjacent.bin` into malloc'd host arrays.
 * Replaces graph::graph (Without-graph-partition/graph.hpp:18-67) and fsize
 * (Without-graph-partition/comm.h:26-32): n = bytes(begin)/8 - 1, m = bytes(adj)/4, with the
 * size checks the reference omits.  Free with trust_tc_free_host. */
int trust_tc_load_folder(const char *folder, int64_t **begin, int32_t **adj, int64_t *n, int64_t *m);
/* Write a CSR as begin.bin/adjacent.bin (the format Preprocess/preprocess_outdegree.cpp:205-221 writes). */
int trust_tc_save_folder(const char *folder, const int64_t *begin, const int32_t *adj, int64_t n,
                         int64_t m);
void trust_tc_free_host(void *p);

/* The reference operator end to end: load folder, validate, copy, count.  Replaces
 * Triangle_count (Without-graph-partition/TC.cu:602-731). */
int trust_tc_count_folder(const char *folder, const trust_tc_opts *opts, trust_tc_result *result);

/* Partitioned operator as a one-GPU tile loop.  `folder` holds partition<i>_<j>/ tiles in the
 * format of Preprocess/partition.cpp:72-121; all parts x parts x parts tile jobs (i,j,k) run on
 * this GPU.  Replaces the partitioned Triangle_count (With-graph-partition/TC.cu:976-1157), which
 * runs one (i,j,k) job per MPI rank.  For simple oriented graphs the total equals the
 * unpartitioned count. */
int trust_tc_count_partitioned(const char *folder, int parts, const trust_tc_opts *opts,
                               trust_tc_result *result);
/* The same tile loop for a device-resident CSR: the GPU splits it into parts x parts tiles (the
 * layout of Preprocess/partition.cpp:72-121, in pinned host memory), then the (i,j,k) jobs run
 * with the tiles streamed into a device cache of at most device_budget_bytes (0 = 80 % of free
 * memory): the larger-than-HBM mode, exercised on any graph by a small budget.  parts <= 32.
 * result->call_seconds spans the job loop including the tile copies (the partition excluded). */
int trust_tc_count_tiles_device(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m, int parts,
                                size_t device_budget_bytes, const trust_tc_opts *opts, trust_tc_result *r);

/* Split a CSR into parts x parts tiles (row class v%parts, column class w%parts, local id w/parts)
 * and write them as partition<i>_<j>/begin.bin,adjacent.bin under `folder`.  Follows
 * Preprocess/partition.cpp:72-121 for the tile contents (map/division files are not written:
 * the tile loop schedules rows itself). */
int trust_tc_partition_folder(const char *folder, const int64_t *begin, const int32_t *adj,
                              int64_t n, int64_t m, int parts);

/* ---- GPU preprocessing: edge pairs -> oriented CSR -------------------------------------- */
/* Build the oriented CSR from `npairs` (u,v) int32 pairs on the device (2*npairs ints, u at
 * even index).  Steps: drop self-loops, symmetrise, drop duplicates, drop vertices without
 * edges, orient each edge from lower to higher (degree, id), renumber by out-degree descending
 * (ties by compacted id), rows sorted ascending.  Replaces Preprocess/fromDirectToUndirect.cpp
 * :29-119 and Preprocess/preprocess_outdegree.cpp:79-222 (ties there follow std::sort order).
 * Outputs are device arrays allocated by the library; free with trust_tc_free_device.
 * `id_bound` is an exclusive upper bound on input ids. */
int trust_tc_build_csr_device(trust_tc_ctx *ctx, const int32_t *d_pairs, int64_t npairs,
                              int64_t id_bound, int64_t **d_begin, int32_t **d_adj, int64_t *n,
                              int64_t *m);
/* The same for a batch: pairs of many graphs in one array, graph g owning original ids
 * [graph_vbeg[g], graph_vbeg[g+1]) (host array of num_graphs+1 entries, graph_vbeg[0] = 0).  New
 * ids keep the original order (no out-degree renumbering), so every graph stays a contiguous
 * range of rows; graph_vbeg_out (host, num_graphs+1) receives those ranges.  The result is the
 * input of trust_tc_batch_create.  No counterpart in the reference (one graph per run). */
int trust_tc_build_batch_device(trust_tc_ctx *ctx, const int32_t *d_pairs, int64_t npairs,
                                const int64_t *graph_vbeg, int64_t num_graphs, int64_t **d_begin,
                                int32_t **d_adj, int64_t *n, int64_t *m, int64_t *graph_vbeg_out);
void trust_tc_free_device(void *p);
/* Copy `bytes` between any two buffers the CUDA runtime can address (cudaMemcpyDefault); lets a
 * caller that owns memory through another allocator take over library-allocated outputs. */
int trust_tc_copy(void *dst, const void *src, size_t bytes);

/* ---- deterministic synthetic graphs (counter-based RNG: identical on every host and GPU) -- */
/* R-MAT: npairs = edge_factor << scale pairs with quadrant probabilities a,b,c (d = 1-a-b-c). */
int trust_tc_gen_rmat_device(trust_tc_ctx *ctx, int scale, int64_t npairs, double a, double b,
                             double c, uint64_t seed, int32_t *d_pairs);
/* Chung-Lu: n vertices, expected degree w_i = w_max * (1 + i/i0)^(-1/(gamma-1)), i0 chosen so
 * that sum w = 2*target_edges; draws npairs endpoint pairs proportional to w. */
int trust_tc_gen_chung_lu_device(trust_tc_ctx *ctx, int64_t n, double gamma, double w_max,
                                 int64_t target_edges, int64_t npairs, uint64_t seed,
                                 int32_t *d_pairs);
/* Barabasi-Albert preferential attachment: n vertices, d edges each (n*d pairs; vertex 0's d
 * pairs are self loops, the seed graph), by the endpoint-copy method (Batagelj & Brandes 2005,
 * per edge as in Sanders & Schulz 2016). */
int trust_tc_gen_ba_device(trust_tc_ctx *ctx, int64_t n, int d, uint64_t seed, int32_t *d_pairs);
/* The Chung-Lu cumulative endpoint table used by trust_tc_gen_chung_lu_device (host, n entries,
 * scaled to 2^63).  Returns i0. */
double trust_tc_chung_lu_table(int64_t n, double gamma, double w_max, int64_t target_edges, uint64_t *cdf);
/* Erdos-Renyi G(n, npairs): uniform endpoint pairs. */
int trust_tc_gen_er_device(trust_tc_ctx *ctx, int64_t n, int64_t npairs, uint64_t seed,
                           int32_t *d_pairs);

/* Autotuner for one graph (device CSR, opts->ptr_kind = TRUST_TC_DEVICE): times the counting call
 * `repeats` times per candidate and keeps the fastest, by coordinate descent from `base` over
 * the schedule (learned / tuned / plain, the last winning on some small graphs), then threads
 * per CTA (128/256/512/1024), warp-class bound (64/128/256, and the default), queue chunk
 * (4/8/16) and, when
 * the graph has rows above the CTA table, hub_cluster (0/1/2/4/-1).  *best receives the chosen
 * options (pass them to trust_tc_count_csr), *best_ms their median call time.  Every candidate
 * must give the same count (else TRUST_TC_E_DEVICE).  time_budget_s > 0 bounds the search: no new
 * candidate starts once the calls made so far add up to that much time (0 = no bound; the
 * candidates are tried in the order above, so a bound keeps the ones that matter most).  No
 * counterpart in the reference, whose threads/blocks/chunk come from argv
 * (Without-graph-partition/mpi_main.cpp:78-81). */
int trust_tc_autotune(trust_tc_ctx *ctx, const int64_t *begin, const int32_t *adj, int64_t n, int64_t m,
                      const trust_tc_opts *base, int repeats, double time_budget_s, trust_tc_opts *best,
                      double *best_ms);

/* ---- batches: many graphs counted by one CUDA-graph launch -------------------------------
 * A batch is the disjoint union of many oriented graphs in one device CSR (ids global), graph g
 * owning rows [graph_vbeg[g], graph_vbeg[g+1]) and no arc leaving its graph (build it with
 * trust_tc_build_batch_device).  Graphs fall into TRUST_TC_BATCH_CLASSES size classes by vertex
 * count ([0,512), [512,4096), [4096,32768), [32768,...)), each with its own warp-class bound;
 * every row of every graph is then counted by one persistent kernel launch.  Validation,
 * classification, list offsets, that launch and the readback of the per-graph counts are captured
 * in one CUDA graph at creation and replayed by every run.  No counterpart in the reference, which
 * counts one graph per run (Without-graph-partition/mpi_main.cpp:75-119); the per-graph counts
 * equal its counts. */
#define TRUST_TC_BATCH_CLASSES 4
typedef struct trust_tc_batch_class {
  int threads_per_block; /* 64..1024, multiple of 32 (default 256); the one launch uses the value
                            of the largest size class present                                 */
  int warp_max_degree;   /* out-degree above which a vertex gets a whole CTA (default 128)     */
  int chunk;             /* vertices per queue claim (default 8); as threads_per_block        */
} trust_tc_batch_class;
typedef struct trust_tc_batch trust_tc_batch;

/* Validates the union (offsets, ids, no arc across graphs), then plans and captures the job.
 * The batch borrows d_begin / d_adj and the context; graph_vbeg is a host array. */
int trust_tc_batch_create(trust_tc_ctx *ctx, const int64_t *d_begin, const int32_t *d_adj, int64_t n,
                          int64_t m, const int64_t *graph_vbeg, int64_t num_graphs, trust_tc_batch **out);
void trust_tc_batch_destroy(trust_tc_batch *batch);
/* graphs, vertices and largest out-degree of every size class (TRUST_TC_BATCH_CLASSES each) */
int trust_tc_batch_info(const trust_tc_batch *batch, int64_t *graphs, int64_t *vertices,
                        int32_t *max_out_degree);
int trust_tc_batch_get_class(const trust_tc_batch *batch, int size_class, trust_tc_batch_class *cfg);
/* sets one size class's launch parameters and re-captures the job */
int trust_tc_batch_set_class(trust_tc_batch *batch, int size_class, const trust_tc_batch_class *cfg);
/* Times the counting launch under each candidate (threads 128/256/512/1024 x warp bound 64/128 x
 * chunk 2/4/8/16, the same for every size class, `repeats` runs each, fastest kept), then each
 * size class's warp bound on its own, keeps the fastest and re-captures the job; *best_ms = the
 * chosen launch's time. */
int trust_tc_batch_autotune(trust_tc_batch *batch, int repeats, double *best_ms);
/* One launch of the captured job on `stream` (waits for it).  counts: host array of num_graphs
 * uint64 per-graph triangle counts (or NULL); result: totals, call_seconds = the graph's
 * CUDA-event time. */
int trust_tc_batch_run(trust_tc_batch *batch, void *stream, uint64_t *counts, trust_tc_result *result);

/* ---- the learned schedule's per-vertex cost model ----------------------------------------
 * An MLP, 8 fp32 features -> 32 -> 32 -> 1 (ReLU), predicting log2 of a vertex's counting cycles.
 * Features of a vertex v with out-degree d(v) >= 2 (trust_tc_vertex_features):
 *   log2(1+d(v)), log2(1+W), log2(1+Wmin), log2(1+max d(u)), log2(1+#arcs with d(u) > d(v)),
 *   log2(1+W/d(v)), schedule class (0..7), log2(table slots)
 * where W = sum over arcs (v,u) of d(u) and Wmin = sum of min(d(u), d(v)).  Trained on the GPU by
 * this library's forward/backward/Adam kernels on cycles recorded with opts.record_cycles.
 * No counterpart in the reference (its schedule is the fixed USE_CTA/USE_WARP split). */
int trust_tc_model_floats(void);
int trust_tc_model_init(float *model, uint64_t seed);
/* mean-squared-error gradient at `model` over device arrays x (n x 8) and y (n) -> host grad */
int trust_tc_model_grad(const float *d_x, const float *d_y, int64_t n, const float *model, float *grad,
                        float *loss);
/* normalise from the data, then `epochs` passes of mini-batch Adam; model is host in/out */
int trust_tc_model_train(const float *d_x, const float *d_y, int64_t n, int epochs, int batch, float lr,
                         float *model, float *loss);
int trust_tc_model_predict(const float *d_x, int64_t n, const float *model, float *d_out);
/* the model compiled into the library (trained on the generated training graphs) */
int trust_tc_model_default(float *model);
/* per-vertex features of a device CSR: d_features n x 8 (zeros for out-degree < 2); the schedule
 * class is the tuned schedule's */
int trust_tc_vertex_features(trust_tc_ctx *ctx, const int64_t *d_begin, const int32_t *d_adj, int64_t n,
                             int64_t m, float *d_features);

#ifdef __cplusplus
}
#endif
#endif /* TRUST_TC_H */

// tc_shim.cpp — Triangle_count with the reference's C++ signature (Without-graph-partition/TC.cuh:10
// and With-graph-partition/TC.cuh:10) implemented over the C ABI.
#include <stdio.h>
#include <stdlib.h>

#include "../../include/trust_tc.h"
#include "../../include/trust_tc_shim.h"

static struct arguments shim_finish(int rc, const trust_tc_result &r, struct arguments args) {
  if (rc != TRUST_TC_OK) {
    // the reference prints the CUDA error and exits (Without-graph-partition/herror.h:1-8)
    printf("\n%s %s in Triangle_count\n", trust_tc_strerror(rc), trust_tc_last_cuda_error());
    exit(EXIT_FAILURE);
  }
  args.time = r.kernel_seconds;
  args.count = (long long)r.triangles;
  args.edge_count = (int)r.edges;
  args.degree = r.vertices ? (int)(r.edges / r.vertices) : 0;  // TC.cu:728
  args.vertices = (int)r.vertices;
  return args;
}

static void shim_opts(trust_tc_opts *o, int n_threads, int n_blocks, int chunk_size) {
  trust_tc_opts_init(o);
  o->threads_per_block = n_threads;
  o->blocks = n_blocks;
  o->chunk = chunk_size;
}

struct arguments Triangle_count(int rank, char name[100], struct arguments args, int total_process, int n_threads,
                                int n_blocks, int chunk_size) {
  (void)total_process;
  trust_tc_opts o;
  shim_opts(&o, n_threads, n_blocks, chunk_size);
  trust_tc_result r = trust_tc_result();
  if (rank > 0) {
    // one GPU: rank 0 already returned the whole count; keep the sizes for the output line
    int64_t *b = nullptr, n = 0, m = 0;
    int32_t *a = nullptr;
    int rc = trust_tc_load_folder(name, &b, &a, &n, &m);
    trust_tc_free_host(b);
    trust_tc_free_host(a);
    r.vertices = n;
    r.edges = m;
    return shim_finish(rc, r, args);
  }
  int rc = trust_tc_count_folder(name, &o, &r);
  return shim_finish(rc, r, args);
}

struct arguments Triangle_count(int rank, char name[100], struct arguments args, int total_process, int n_threads,
                                int n_blocks, int chunk_size, int partition_num) {
  (void)total_process;
  trust_tc_opts o;
  shim_opts(&o, n_threads, n_blocks, chunk_size);
  trust_tc_result r = trust_tc_result();
  if (rank > 0) return shim_finish(TRUST_TC_OK, r, args);
  int rc = trust_tc_count_partitioned(name, partition_num, &o, &r);
  return shim_finish(rc, r, args);
}

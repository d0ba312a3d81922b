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
  int64_t *d_beg = nullptr;
  size_t beg_cap = 0;
  int32_t *d_adj = nullptr;
  size_t adj_cap = 0;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

namespace tc {

// Three CSRs on the device: A rows are hashed, B rows give the arcs (v,u), C rows are probed.
struct DevGraph3 {
  const int64_t *begA, *begB, *begC;
  const int32_t *adjA, *adjB, *adjC;
  int64_t rows;               // rows of A and B
  int64_t rowsC;              // rows of C
  int64_t mA, mB, mC;         // entries of each
  int64_t boundA, boundB, boundC;  // exclusive id bound per CSR (B's ids index rows of C)
  int min_deg;                // rows with fewer entries in A or B are skipped
};

int ctx_init(trust_tc_ctx *c, int device);
void ctx_release(trust_tc_ctx *c);
int ensure(void **p, size_t *cap, size_t bytes);
int count_device(trust_tc_ctx *c, const DevGraph3 &g, const trust_tc_opts &o, bool check_ids,
                 trust_tc_result *r);

}  // namespace tc

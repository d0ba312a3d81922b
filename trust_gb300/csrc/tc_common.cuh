// tc_common.cuh — shared definitions for the sm_103a triangle-counting kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/trust_tc.h"

#define TC_FULL_MASK 0xffffffffu

// Schedule classes.  Index 0 = skipped (out-degree < 2, as the warp loop of
// Without-graph-partition/TC.cu:440 stops there); 1..4 = sub-warp groups of 4/8/16/32 lanes;
// 5 = a warp with several arc rounds; 6 = a CTA with a shared-memory table; 7 = a CTA with a
// table larger than shared memory (cluster / global).
enum {
  TC_CLASS_SKIP = 0,
  TC_CLASS_G4 = 1,
  TC_CLASS_G8 = 2,
  TC_CLASS_G16 = 3,
  TC_CLASS_G32 = 4,
  TC_CLASS_WARP = 5,
  TC_CLASS_CTA = 6,
  TC_CLASS_HUGE = 7,
  TC_NUM_CLASSES = 8
};

// Device status words (written by the kernels, read by the host after the call).
enum {
  TC_DEV_OK = 0,
  TC_DEV_BAD_OFFSETS = 1,
  TC_DEV_BAD_IDS = 2,
  TC_DEV_TOO_LARGE = 4,
  TC_DEV_TABLE_FULL = 8,  // a hash insert found no free slot (cannot happen when sized 2x)
  TC_DEV_WAIT_LIMIT = 16,  // a bounded spin wait ran out
  TC_DEV_UNSORTED = 32     // informational: some row is not strictly increasing
};

// Control block living in device scratch.  One per counting call.
struct TcControl {
  unsigned long long count;           // the u64 triangle count
  unsigned long long wedges;          // sum of probe counts (diagnostic)
  int status;                         // TC_DEV_* bits
  int max_out_degree;
  unsigned long long bad_offset_at;   // first vertex with a bad offset (diagnostic)
  int class_count[TC_NUM_CLASSES];    // list sizes after classification
  int class_cursor[TC_NUM_CLASSES];   // scatter cursors of the classification pass
  int class_next[TC_NUM_CLASSES];     // work-queue heads (atomic chunk claims)
  int class_off[TC_NUM_CLASSES];      // list offsets, when computed on the device (batches)
  unsigned long long long_arcs;       // arcs of rows longer than TC_LONG_ROW (single-graph calls)
  int class_count_alt[TC_NUM_CLASSES];  // small graphs: list sizes under the plain split as well
};
constexpr int TC_LONG_ROW = 128;

#if defined(__CUDACC__)
// Knuth multiplicative hash into a power-of-two table of 2^log2 slots.
__device__ __forceinline__ unsigned tc_hash(unsigned key, int log2) {
  return (key * 0x9E3779B1u) >> (32 - log2);
}

__device__ __forceinline__ unsigned tc_lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int tc_ld_nc(const int32_t *p) { return __ldg(p); }
__device__ __forceinline__ long long tc_ld_nc(const int64_t *p) {
  return __ldg(reinterpret_cast<const long long *>(p));
}

#endif  // __CUDACC__

// Host helpers shared by the translation units.
namespace tc {
int cuda_status(cudaError_t e);  // records the text, returns TRUST_TC_E_CUDA (or OK)
void note_launch(uint64_t k = 1);  // k more kernels launched by the library
}

// After every kernel launch of the library (trust_tc_kernel_launches reports the total).
#define TC_NOTE_LAUNCH() ::tc::note_launch()

#define TC_CUDA_TRY(expr)                              \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return tc::cuda_status(_e); \
  } while (0)

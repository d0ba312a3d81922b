/*
 * ref_tc_driver.c — runs the reference counting kernel (Without-graph-partition/TC.cu
 * dynamic_assign, compiled from source for sm_103a into oracle/_ref/tc_ref_w.cubin by
 * oracle/build_ref.sh) on the GPU.  TEST INFRASTRUCTURE ONLY: a second, independent oracle for
 * the counting kernel and the "reference kernel rebuilt for sm_103a" timing.
 *
 * The host steps restate Triangle_count (Without-graph-partition/TC.cu:602-731) for one rank:
 *   warpfirstvertex = my_binary_search(n, USE_CTA=100, beg) + 1         (:632)
 *   G_INDEX seeds {chunk*blocks*threads/32, chunk*blocks, warpfirst + chunk*blocks*threads/32}
 *                                                                        (:666-669)
 *   BIN_MEM = blocks * 1024 * 100 ints                                   (:608, :682)
 *   dynamic_assign<<<blocks, threads>>>(adj, beg, m, n, BIN_MEM, COUNT, rank 0, 1 process,
 *                                       BUCKET_SIZE 100, T_Group 32, G_INDEX, chunk, warpfirst,
 *                                       gettime, maxcollision)          (:688)
 * Differences, all for memory safety on a shared GPU: the counter is zeroed (the reference
 * relies on fresh cudaMalloc memory, :655), adjacent is followed by 64 zero ints (the kernel
 * reads up to 15 entries past a row end, TC.cu:342-349 and :522-529), the unused timing buffers
 * are one element long, and the caller must first certify the input with orc_trust_check
 * (no bucket beyond 98 entries, class layout, offsets < 2^31) and pass threads == 1024.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define REF_KERNEL "_Z14dynamic_assignPiPliiS_PyiiiiS_iiS1_S1_"

extern int64_t orc_trust_split(const int64_t *beg, int64_t n, int val);

static char g_err[256];
const char *orc_ref_tc_error(void) { return g_err; }

#define CK(x)                                                   \
  do {                                                          \
    CUresult _r = (x);                                          \
    if (_r != CUDA_SUCCESS) {                                   \
      const char *s = 0;                                        \
      cuGetErrorString(_r, &s);                                 \
      strncpy(g_err, s ? s : "cuda driver error", sizeof g_err - 1); \
      rc = (int)_r;                                             \
      goto done;                                                \
    }                                                           \
  } while (0)

/* Returns 0 on success; count and kernel milliseconds (CUDA events around the launch). */
int orc_ref_tc_run(const char *cubin, const int64_t *beg, const int32_t *adj, int64_t n, int64_t m,
                   int threads, int blocks, int chunk, uint64_t *count, float *ms) {
  int rc = 0;
  CUdevice dev;
  CUcontext ctx = 0;
  CUmodule mod = 0;
  CUfunction fn;
  CUdeviceptr d_count = 0, d_tt = 0, d_mc = 0, d_index = 0, d_beg = 0, d_adj = 0, d_bin = 0;
  CUevent e0 = 0, e1 = 0;
  int pushed = 0;
  g_err[0] = 0;
  if (threads != 1024 || blocks <= 0 || chunk <= 0 || m >= ((int64_t)1 << 31) || n >= ((int64_t)1 << 31)) {
    strcpy(g_err, "reference kernel needs threads=1024 and m, n < 2^31");
    return -1;
  }
  CK(cuInit(0));
  {
    int ord = 0;
    CUcontext cur = 0;
    if (cuCtxGetCurrent(&cur) == CUDA_SUCCESS && cur) {
      CK(cuCtxGetDevice(&dev));
    } else {
      CK(cuDeviceGet(&dev, ord));
    }
  }
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxPushCurrent(ctx));
  pushed = 1;
  CK(cuModuleLoad(&mod, cubin));
  CK(cuModuleGetFunction(&fn, mod, REF_KERNEL));
  {
    int warpfirst = (int)(orc_trust_split(beg, n, 100) + 1);
    int seeds[3];
    seeds[0] = chunk * blocks * threads / 32;
    seeds[1] = chunk * (blocks * 1 + 0);
    seeds[2] = warpfirst + chunk * (blocks * threads / 32 * 1 + 0);
    size_t bin_ints = (size_t)blocks * 1024 * 100;
    CK(cuMemAlloc(&d_count, 10 * sizeof(uint64_t)));
    CK(cuMemsetD8(d_count, 0, 10 * sizeof(uint64_t)));
    CK(cuMemAlloc(&d_tt, sizeof(uint64_t)));
    CK(cuMemAlloc(&d_mc, sizeof(uint64_t)));
    CK(cuMemAlloc(&d_index, 3 * sizeof(int)));
    CK(cuMemcpyHtoD(d_index, seeds, sizeof seeds));
    CK(cuMemAlloc(&d_beg, (size_t)(n + 1) * sizeof(int64_t)));
    CK(cuMemcpyHtoD(d_beg, beg, (size_t)(n + 1) * sizeof(int64_t)));
    CK(cuMemAlloc(&d_adj, (size_t)(m + 64) * sizeof(int32_t)));
    CK(cuMemsetD8(d_adj, 0, (size_t)(m + 64) * sizeof(int32_t)));
    if (m) CK(cuMemcpyHtoD(d_adj, adj, (size_t)m * sizeof(int32_t)));
    CK(cuMemAlloc(&d_bin, bin_ints * sizeof(int)));
    int edge_count = (int)m, vertex_count = (int)n, rank = 0, total_process = 1, bucket = 100, tgroup = 32;
    void *args[15] = {&d_adj, &d_beg, &edge_count, &vertex_count, &d_bin, &d_count, &rank, &total_process,
                      &bucket, &tgroup, &d_index, &chunk, &warpfirst, &d_tt, &d_mc};
    CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    CK(cuEventRecord(e0, 0));
    CK(cuLaunchKernel(fn, (unsigned)blocks, 1, 1, (unsigned)threads, 1, 1, 0, 0, args, 0));
    CK(cuEventRecord(e1, 0));
    CK(cuEventSynchronize(e1));
    CK(cuEventElapsedTime(ms, e0, e1));
    uint64_t host_count[10];
    CK(cuMemcpyDtoH(host_count, d_count, sizeof host_count));
    *count = host_count[0];
  }
done:
  if (e0) cuEventDestroy(e0);
  if (e1) cuEventDestroy(e1);
  if (d_bin) cuMemFree(d_bin);
  if (d_adj) cuMemFree(d_adj);
  if (d_beg) cuMemFree(d_beg);
  if (d_index) cuMemFree(d_index);
  if (d_mc) cuMemFree(d_mc);
  if (d_tt) cuMemFree(d_tt);
  if (d_count) cuMemFree(d_count);
  if (mod) cuModuleUnload(mod);
  if (pushed) cuCtxPopCurrent(&ctx);
  if (ctx) cuDevicePrimaryCtxRelease(dev);
  return rc;
}

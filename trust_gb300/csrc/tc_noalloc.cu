// tc_noalloc.cu — a counting entry point that allocates nothing.
//
// Who needs it: callers that may not allocate GPU memory while they count.  Examples are a host
// whose device memory is handed out by its own pool under a fixed budget (a database or stream
// processor that forbids outside cudaMalloc), code running where cudaMalloc's implicit device
// synchronisation would stall other work sharing the GPU, and callers that must not fail halfway
// through for lack of memory.  trust_tc_count_csr needs scratch (a control block and per-class
// vertex lists) that its context allocates; this variant takes that scratch from one fixed array
// in the library's device image instead.
//
// The array, g_noalloc_scratch, is TC_NOALLOC_SCRATCH_BYTES (16 MiB) of device memory that every
// GPU which loads the library holds until the process exits.  Host code cannot use the symbol's
// name as a device address, so the first call on each device looks its address up with
// cudaGetSymbolAddress (with that device current) and keeps it for the life of the process; make
// that first call before any stream capture.  The kept address belongs to the device's primary
// context: after cudaDeviceReset on that device the process must not call this entry point again.
// All calls share the array and leave their contents in it; the control block at its start is
// cleared on the stream at the start of every call.  Calls that overlap on the GPU (several
// streams or threads at once) race on the array and must be serialised by the caller.  Each call
// synchronises its stream twice (after classification, to size the class lists, and after the
// count) and returns with the caller's current device unchanged.
#include <algorithm>
#include <mutex>

#include "tc_count.h"

namespace {

constexpr size_t TC_NOALLOC_SCRATCH_BYTES = (size_t)16 << 20;
constexpr size_t TC_NOALLOC_LISTS_OFFSET = 256;  // control block first, lists 256-byte aligned
constexpr int64_t TC_NOALLOC_MAX_ROWS = (int64_t)((TC_NOALLOC_SCRATCH_BYTES - TC_NOALLOC_LISTS_OFFSET) / sizeof(int));
constexpr int TC_NOALLOC_MAX_DEVICES = 64;

static_assert(sizeof(TcControl) <= TC_NOALLOC_LISTS_OFFSET, "control block must fit before the lists");

__device__ __align__(256) unsigned char g_noalloc_scratch[TC_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[TC_NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on `device` (which must be current); looked up once.
int noalloc_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= TC_NOALLOC_MAX_DEVICES) return TRUST_TC_E_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return tc::cuda_status(e);
    g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_noalloc_ptr[device];
  return TRUST_TC_OK;
}

int ceil_log2_i64(int64_t x) {
  int l = 0;
  while (((int64_t)1 << l) < x) ++l;
  return l;
}

}  // namespace

// Puts the caller's current device back when the call returns.
struct DeviceRestore {
  int prev = -1;
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

static int count_noalloc(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                         const trust_tc_opts &o, trust_tc_result *r);

extern "C" int trust_tc_count_csr_noalloc(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                                          const trust_tc_opts *opts, trust_tc_result *r) {
  if (!d_begin || !r || n < 0 || m < 0 || (m > 0 && !d_adj)) return TRUST_TC_E_ARG;
  if (n > TC_NOALLOC_MAX_ROWS || m >= ((int64_t)1 << 31)) return TRUST_TC_E_TOO_LARGE;
  trust_tc_opts o;
  if (opts) o = *opts; else trust_tc_opts_init(&o);
  if (o.ptr_kind != TRUST_TC_DEVICE) return TRUST_TC_E_UNSUPPORTED;
  // per-vertex cycles would be written into a caller array this variant does not clear: refused
  // rather than silently left untouched
  if (o.record_cycles) return TRUST_TC_E_UNSUPPORTED;
  if (o.row_begin || o.row_end) return TRUST_TC_E_UNSUPPORTED;  // row ranges: trust_tc_count_csr only
  uint64_t *cycles = r->vertex_cycles;
  *r = trust_tc_result();
  r->vertex_cycles = cycles;
  r->vertices = n;
  r->edges = m;
  DeviceRestore restore;
  TC_CUDA_TRY(cudaGetDevice(&restore.prev));
  return count_noalloc(d_begin, d_adj, n, m, o, r);
}

static int count_noalloc(const int64_t *d_begin, const int32_t *d_adj, int64_t n, int64_t m,
                         const trust_tc_opts &o, trust_tc_result *r) {
  int device = o.device;
  if (device < 0) TC_CUDA_TRY(cudaGetDevice(&device));
  TC_CUDA_TRY(cudaSetDevice(device));
  unsigned char *scratch = nullptr;
  int rc = noalloc_scratch(device, &scratch);
  if (rc) return rc;
  // launch configuration: the same defaults and limits as trust_tc_count_csr
  int num_sms = 0, smem_optin = 0;
  TC_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
  TC_CUDA_TRY(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  const int threads = o.threads_per_block > 0 ? o.threads_per_block : 256;
  const int warp_max =
      o.warp_max_degree > 0 ? o.warp_max_degree : (o.schedule == TRUST_TC_SCHED_PLAIN ? 100 : 512);
  const int want_cta = o.block_max_degree > 0 ? o.block_max_degree : 4096;
  if (threads % 32 || threads < 64 || threads > 1024 || warp_max < 32 || warp_max > 4096 || want_cta < warp_max)
    return TRUST_TC_E_ARG;
  const int cta_log2 = std::max(ceil_log2_i64(2 * (int64_t)want_cta), 6);
  const int warp_slots = 1 << std::max(ceil_log2_i64(2 * (int64_t)warp_max), 7);
  const size_t smem = std::max((size_t)4 << cta_log2, (size_t)4 * warp_slots * (threads / 32));
  if (smem > (size_t)smem_optin) return TRUST_TC_E_ARG;
  const int cta_max = 1 << (cta_log2 - 1);
  int per_sm = 0;
  rc = tc::count_kernel_occupancy(true, threads, smem, &per_sm);
  if (rc) return rc;
  if (per_sm < 1) return TRUST_TC_E_ARG;
  rc = tc::set_count_kernel_carveout(true, threads, smem, per_sm);
  if (rc) return rc;
  const int blocks = o.blocks > 0 ? o.blocks : num_sms * per_sm;

  cudaStream_t st = (cudaStream_t)o.stream;
  TcControl *ctl = reinterpret_cast<TcControl *>(scratch);
  int *lists = reinterpret_cast<int *>(scratch + TC_NOALLOC_LISTS_OFFSET);
  TC_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(TcControl), st));
  rc = tc::launch_check(d_begin, d_adj, n, m, n, o.validate >= TRUST_TC_VALIDATE_FULL, ctl, num_sms, st);
  if (rc) return rc;
  tc::ListOffsets off{};
  rc = tc::launch_classify(0, d_begin, d_begin, n, 2, warp_max, cta_max, ctl, lists, off, num_sms, st, o.schedule);
  if (rc) return rc;
  TcControl h;
  TC_CUDA_TRY(cudaMemcpyAsync(&h, ctl, sizeof h, cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  if (h.status & TC_DEV_BAD_OFFSETS) return TRUST_TC_E_OFFSETS;
  if (h.status & TC_DEV_TOO_LARGE) return TRUST_TC_E_TOO_LARGE;
  if (h.status & TC_DEV_BAD_IDS) return TRUST_TC_E_IDS;
  // a vertex above the CTA table size would need a spill table: not available without allocating
  if (h.class_count[TC_CLASS_HUGE] > 0) return TRUST_TC_E_TOO_LARGE;
  int64_t total = 0;
  for (int k = TC_CLASS_SKIP + 1; k < TC_NUM_CLASSES; ++k) {
    off.off[k] = (int)total;
    total += h.class_count[k];
  }
  rc = tc::launch_classify(1, d_begin, d_begin, n, 2, warp_max, cta_max, ctl, lists, off, num_sms, st, o.schedule);
  if (rc) return rc;
  tc::CountArgs a{};
  a.begA = a.begB = a.begC = d_begin;
  a.adjA = a.adjB = a.adjC = d_adj;
  a.rows = n;
  a.lists = lists;
  a.off = off;
  a.ctl = ctl;
  a.warp_slots = warp_slots;
  a.chunk = o.chunk > 0 ? o.chunk : 8;
  rc = tc::launch_count(true, a, blocks, threads, smem, st);
  if (rc) return rc;
  TcControl done;
  TC_CUDA_TRY(cudaMemcpyAsync(&done, ctl, sizeof done, cudaMemcpyDeviceToHost, st));
  TC_CUDA_TRY(cudaStreamSynchronize(st));
  if (done.status & TC_DEV_TABLE_FULL) return TRUST_TC_E_DEVICE;
  r->triangles = done.count;
  r->wedges = (int64_t)done.wedges;
  r->max_out_degree = done.max_out_degree;
  for (int k = 0; k < TC_NUM_CLASSES; ++k) r->class_sizes[k] = h.class_count[k];
  r->direction_split = 0;
  r->split_saving_ms = 0.f;
  return TRUST_TC_OK;
}

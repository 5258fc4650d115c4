// wfa_noalloc.cu -- batch alignment that allocates no memory.
//
// Some callers cannot let a library allocate GPU memory: processes whose
// device memory is owned by a framework pool or planned to the byte up front
// (long-running servers, plugins hosted inside another runtime), and code
// paths where cudaMalloc's implicit device-wide synchronisation is not
// acceptable.  For them, wf2g_noalloc_align() runs the same alignment kernel
// with its scratch (wavefront rows, back-trace table and choice bytes, work
// queue) carved out of one fixed array in device memory that is part of this
// library image.  Every GPU that loads the library holds that array until the
// process exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "wfa_engine.h"
#include "wfa_kernels.cuh"

namespace wf2g {
extern "C" void* wf2g_kernel_ptr(int a2p, int cigar, int enc, int off_bytes, int heur, int wide,
                                 int ef, int lin);
extern "C" int wf2g_seq_bytes(int enc, int max_len);
}  // namespace wf2g

using namespace wf2g;

// The fixed scratch: 64 MiB per device, shared by every call.
static constexpr size_t kNoAllocBytes = size_t(64) << 20;
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocBytes];

// Largest pattern/text length this entry point accepts, and the back-trace
// bytes each warp may use (a pair needing more reports WF_STATUS_OOM).
static constexpr int kNoAllocMaxLen = 2048;
static constexpr int64_t kNoAllocBitsPerWarp = int64_t(512) << 10;
static constexpr int kMaxDevices = 64;

// Host code cannot use the array's name as a device address: resolve it with
// cudaGetSymbolAddress, with the device current.  The address belongs to the
// CUDA context that loaded the module: after cudaDeviceReset (or any reset of
// the primary context) the module is loaded again and the array may move, so
// the cached address is keyed by the context's unique id (cuCtxGetId) and
// resolved again when that id changes.
static std::mutex g_setup_mutex;
static uint8_t* g_scratch_ptr[kMaxDevices];
static unsigned long long g_scratch_ctx[kMaxDevices];

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);
static PfnCtxGetCurrent g_ctx_get_current = nullptr;
static PfnCtxGetId g_ctx_get_id = nullptr;
static std::once_flag g_driver_once;

// Unique id of the calling thread's current context: 0 on success, 1 when no
// context is current yet, -1 when the driver entry points are unavailable.
static int current_context_id(unsigned long long* id) {
  std::call_once(g_driver_once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_ctx_get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_ctx_get_id = (PfnCtxGetId)f;
    cudaGetLastError();
  });
  if (!g_ctx_get_current || !g_ctx_get_id) return -1;
  CUcontext c = nullptr;
  if (g_ctx_get_current(&c) != CUDA_SUCCESS) return -1;
  if (!c) return 1;
  return g_ctx_get_id(c, id) == CUDA_SUCCESS ? 0 : -1;
}

static uint8_t* scratch_for_current_device(int* err) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    *err = -1;  // WF2G_ERR_NO_GPU
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long id = 0;
  int have_id = current_context_id(&id);
  if (have_id == 0 && g_scratch_ptr[dev] && g_scratch_ctx[dev] == id) return g_scratch_ptr[dev];
  void* ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || ptr == nullptr) {
    fprintf(stderr, "[wfa2gpu] no-alloc scratch: cudaGetSymbolAddress failed: %s\n",
            cudaGetErrorString(e));
    cudaGetLastError();
    *err = -4;  // WF2G_ERR_CUDA
    return nullptr;
  }
  // the lookup initialises the runtime's context if none was current
  if (have_id == 1) have_id = current_context_id(&id);
  // without a context id nothing is cached: the address is looked up per call
  g_scratch_ptr[dev] = have_id == 0 ? (uint8_t*)ptr : nullptr;
  g_scratch_ctx[dev] = id;
  return (uint8_t*)ptr;
}

extern "C" int wf2g_noalloc_align(const wf2g_cfg_t* cfg, int n, const char* d_seqs,
                                  const int64_t* d_poff, const int32_t* d_plen,
                                  const int64_t* d_toff, const int32_t* d_tlen, int max_len,
                                  int32_t* d_scores, int32_t* d_status, char* d_ops,
                                  const int64_t* d_opsoff, int32_t* d_opslen, void* stream) {
  if (!cfg || n < 0) return -3;  // WF2G_ERR_ARGS
  if (max_len > kNoAllocMaxLen || max_len < 0) {
    fprintf(stderr,
            "[wfa2gpu] wavefront_align_batch_device_noalloc: max_sequence_length %d exceeds "
            "the fixed-scratch limit of %d\n",
            max_len, kNoAllocMaxLen);
    return -3;  // WF2G_ERR_ARGS
  }
  if (cfg->metric != 3 && cfg->metric != 4) return -2;  // WF2G_ERR_CONFIG (gap-affine metrics only)
  if (cfg->ultralow) return -2;  // BiWFA allocates per recursion level
  if (cfg->endsfree) return -2;  // the ends-free kernels are not in the fixed-scratch set
  if (cfg->heur & ~wf2g::kHsWfadaptive) return -2;  // wf-adaptive or none only
  const bool cigar = !cfg->score_only;
  if (cigar && (!d_ops || !d_opsoff || !d_opslen)) return -3;
  int err = 0;
  uint8_t* const base = scratch_for_current_device(&err);
  if (!base) return err;
  if (n == 0) return 0;
  const int L = std::max(max_len, 1);
  cudaStream_t st = (cudaStream_t)stream;

  // penalties and ring geometry (the same layout the batch engine uses)
  KParams kp;
  memset(&kp, 0, sizeof(kp));
  kp.metric = cfg->metric;
  Penalties& pen = kp.pen;
  pen.match = cfg->match;
  pen.x = cfg->x;
  pen.o1 = cfg->o1;
  pen.e1 = cfg->e1;
  pen.o2 = cfg->metric == 4 ? cfg->o2 : 0;
  pen.e2 = cfg->metric == 4 ? cfg->e2 : 1;
  int indel = cfg->o1 + cfg->e1;
  if (cfg->metric == 4) indel = std::max(indel, cfg->o2 + cfg->e2);
  pen.R = std::max(indel, cfg->x) + 1;
  pen.RI1 = cfg->e1 + 1;
  pen.RI2 = cfg->metric == 4 ? cfg->e2 + 1 : 1;
  const int nrows = cfg->metric == 4 ? pen.R + 2 * pen.RI1 + 2 * pen.RI2 : pen.R + 2 * pen.RI1;
  int64_t bound = (int64_t)cfg->x * L + cfg->o1 + (int64_t)cfg->e1 * L;
  if (cfg->metric == 4) bound = std::max<int64_t>(bound, (int64_t)cfg->x * L + cfg->o2 + (int64_t)cfg->e2 * L);
  kp.table_cap = (int)(bound + 9);
  kp.max_steps = cfg->max_steps;
  kp.heur = cfg->heur;
  kp.h_min_len = cfg->h_min_len;
  kp.h_max_dist = cfg->h_max_dist;
  kp.h_steps = cfg->h_steps;
  kp.seqs = (const uint8_t*)d_seqs;
  kp.p_off = d_poff;
  kp.p_len = d_plen;
  kp.t_off = d_toff;
  kp.t_len = d_tlen;
  kp.n_items = n;
  kp.final_pass = 1;  // one pass: a pair that outgrows its slice reports WF_STATUS_OOM
  kp.scores = d_scores;
  kp.status = d_status;
  kp.ops = (uint8_t*)d_ops;
  kp.ops_off = d_opsoff;
  kp.ops_len = d_opslen;
  kp.max_len = L;
  kp.kofs = L + 2;
  kp.row_stride = ((2 * L + 6) + 63) & ~63;
  kp.ring_bytes = (((int64_t)(nrows + 1) * kp.row_stride * 2) + 255) & ~int64_t(255);
  const int seq_bytes = wf2g_seq_bytes(8, L);
  kp.seq_in_smem = 1;
  kp.smem_per_group = (int)(((int64_t)seq_bytes + (int64_t)nrows * 16 + 15) & ~int64_t(15));
  kp.bits_cap = cigar ? kNoAllocBitsPerWarp : 0;
  kp.gscratch_per_group =
      (kp.ring_bytes + (cigar ? (int64_t)kp.table_cap * kBtRowBytes + kp.bits_cap : 0) + 255) &
      ~int64_t(255);

  // the array: [control: 256 bytes][per-warp slices]
  const int64_t avail = (int64_t)kNoAllocBytes - 256;
  const int64_t warps_fit = avail / kp.gscratch_per_group;
  if (warps_fit < 1) {
    fprintf(stderr,
            "[wfa2gpu] wavefront_align_batch_device_noalloc: one warp's scratch (%lld bytes) "
            "exceeds the fixed %zu-byte array for these penalties\n",
            (long long)kp.gscratch_per_group, kNoAllocBytes);
    return -3;  // WF2G_ERR_ARGS
  }
  int wpc = (int)std::min<int64_t>(8, warps_fit);
  const size_t smem = (size_t)kp.smem_per_group * wpc;
  if (smem > 48 * 1024) wpc = std::max(1, (int)((48 * 1024) / kp.smem_per_group));
  int blocks = (int)std::min<int64_t>(warps_fit / wpc, ((int64_t)n + wpc - 1) / wpc);
  blocks = std::max(blocks, 1);
  int32_t* const queue = (int32_t*)base;  // the only value that must start at zero
  kp.queue = queue;
  kp.gscratch = base + 256;
  // calls share the array: clear the queue head left by the previous call
  if (cudaMemsetAsync(queue, 0, sizeof(int32_t), st) != cudaSuccess) {
    cudaGetLastError();
    return -4;
  }
  void* fn = wf2g_kernel_ptr(cfg->metric == 4, cigar, 8, 2, cfg->heur, 0, 0, 0);
  void* args[] = {(void*)&kp};
  const cudaError_t e = cudaLaunchKernel(fn, dim3(blocks), dim3(32 * wpc), args,
                                         (size_t)kp.smem_per_group * wpc, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] no-alloc launch failed: %s\n", cudaGetErrorString(e));
    cudaGetLastError();  // the failure is reported here, not left pending for the caller
    return -4;           // WF2G_ERR_CUDA
  }
  return 0;
}

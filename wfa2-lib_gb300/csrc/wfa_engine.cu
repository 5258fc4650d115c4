// wfa_engine.cu -- host side of the GB300 wavefront aligner: device buffers,
// pass planning and kernel launches behind the C interface of wfa_engine.h.
//
// A batch runs in two passes, both persistent kernels that pull pairs from a
// device work queue (no host round trip between them):
//   pass 1  2-bit packed sequences, wavefront ring in shared memory, ring
//           width sized for the common case; pairs whose wavefront outgrows
//           the ring, whose back-trace outgrows the warp's choice-byte slice,
//           or that hold non-ACGT bytes are appended to a retry list;
//   pass 2  8-bit sequences, ring in a private global-memory slice wide enough
//           for any wavefront of the batch (plen+tlen+3 diagonals); runs only
//           over the retry list and reports a remaining overflow as
//           WF_STATUS_OOM.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "wfa_engine.h"
#include "wfa_kernels.cuh"

// WF2G_ERR_* values of include/wfa2gpu.h
#define WF2G_OK_ 0
#define WF2G_ERR_NO_GPU_ -1
#define WF2G_ERR_CONFIG_ -2
#define WF2G_ERR_ARGS_ -3
#define WF2G_ERR_CUDA_ -4
#define WF2G_ERR_OOM_ -5

namespace wf2g {
extern "C" void* wf2g_kernel_ptr(int a2p, int cigar, int enc, int off_bytes);
}

namespace {

using namespace wf2g;

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

int ensure(DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes <= b.cap) return 0;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  const size_t want = bytes + bytes / 4;
  if (cudaMalloc(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  b.cap = want;
  return 0;
}

struct Engine {
  int device = -1;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  // batch buffers (host-input path)
  DevBuf seqs, poff, plen, toff, tlen, scores, status, ops, opsoff, opslen;
  // control
  DevBuf counters;  // [0] queue pass 1, [1] queue pass 2, [2] retry count
  DevBuf retry;
  DevBuf scratch1, scratch2;
};

constexpr int kWarpsPerCta2 = 2;
constexpr int64_t kBits1PerWarp = int64_t(2) << 20;     // pass-1 choice bytes per warp
constexpr int64_t kScratch2Budget = int64_t(24) << 30;  // pass-2 global scratch budget

int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return (v && *v) ? atoi(v) : dflt;
}

int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

struct PassPlan {
  KParams kp;
  int warps_per_cta;
  int blocks;
  size_t smem;
  void* fn;
};

Penalties make_pen(const wf2g_cfg_t& c) {
  Penalties p;
  p.match = c.match;
  p.x = c.x;
  p.o1 = c.o1;
  p.e1 = c.e1;
  p.o2 = c.metric == 4 ? c.o2 : 0;
  p.e2 = c.metric == 4 ? c.e2 : 1;
  // wavefront/wavefront_components.c:81-120: max_score_scope
  int indel = c.o1 + c.e1;
  if (c.metric == 4) indel = std::max(indel, c.o2 + c.e2);
  p.R = std::max(indel, c.x) + 1;
  p.RI1 = c.e1 + 1;
  p.RI2 = c.metric == 4 ? c.e2 + 1 : 1;
  return p;
}

int num_rows(const Penalties& p, bool a2p) { return a2p ? p.R + 2 * p.RI1 + 2 * p.RI2 : p.R + 2 * p.RI1; }

// Upper bound of the alignment score, as the reference sizes its wavefront
// table (wavefront/wavefront_components.c:101-108), for lengths <= max_len.
int score_bound(const wf2g_cfg_t& c, int max_len) {
  int64_t b = (int64_t)c.x * max_len + c.o1 + (int64_t)c.e1 * max_len;
  if (c.metric == 4) b = std::max<int64_t>(b, (int64_t)c.x * max_len + c.o2 + (int64_t)c.e2 * max_len);
  b += 8;
  return (int)std::min<int64_t>(b, INT32_MAX / 4);
}

int launch(Engine* E, const PassPlan& pl, cudaStream_t st) {
  if (pl.blocks <= 0) return 0;
  void* args[] = {(void*)&pl.kp};
  cudaError_t e = cudaLaunchKernel(pl.fn, dim3(pl.blocks), dim3(32 * pl.warps_per_cta), args,
                                   pl.smem, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] kernel launch failed: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  E->launches++;
  return 0;
}

}  // namespace


extern "C" int wf2g_engine_device(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return -1;
  }
  int d = -1;
  if (cudaGetDevice(&d) != cudaSuccess) return -1;
  return d;
}

extern "C" void* wf2g_engine_new(int* err) {
  const int dev = wf2g_engine_device();
  if (dev < 0) {
    if (err) *err = WF2G_ERR_NO_GPU_;
    return nullptr;
  }
  Engine* E = new (std::nothrow) Engine();
  if (!E) {
    if (err) *err = WF2G_ERR_OOM_;
    return nullptr;
  }
  E->device = dev;
  cudaDeviceGetAttribute(&E->num_sms, cudaDevAttrMultiProcessorCount, dev);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  E->smem_optin = (size_t)optin;
  if (cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete E;
    if (err) *err = WF2G_ERR_CUDA_;
    return nullptr;
  }
  // allow every kernel variant the opt-in shared memory
  for (int a2p = 0; a2p < 2; ++a2p)
    for (int cig = 0; cig < 2; ++cig)
      for (int enc = 2; enc <= 8; enc += 6)
        for (int ob = 2; ob <= 4; ob += 2)
          cudaFuncSetAttribute(wf2g_kernel_ptr(a2p, cig, enc, ob),
                               cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (err) *err = WF2G_OK_;
  return E;
}

extern "C" void wf2g_engine_free(void* engine) {
  Engine* E = (Engine*)engine;
  if (!E) return;
  cudaSetDevice(E->device);
  DevBuf* bufs[] = {&E->seqs,   &E->poff,     &E->plen,  &E->toff,     &E->tlen,
                    &E->scores, &E->status,   &E->ops,   &E->opsoff,   &E->opslen,
                    &E->counters, &E->retry,  &E->scratch1, &E->scratch2};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (E->stream) cudaStreamDestroy(E->stream);
  delete E;
}

extern "C" int64_t wf2g_engine_launches(const void* engine) {
  return engine ? ((const Engine*)engine)->launches : 0;
}

static int plan_and_run(Engine* E, const wf2g_cfg_t& cfg, int n, const char* d_seqs,
                        const int64_t* d_poff, const int32_t* d_plen, const int64_t* d_toff,
                        const int32_t* d_tlen, int max_len, int32_t* d_scores,
                        int32_t* d_status, char* d_ops, const int64_t* d_opsoff,
                        int32_t* d_opslen, cudaStream_t st) {
  const bool a2p = (cfg.metric == 4);
  const bool cigar = !cfg.score_only;
  const Penalties pen = make_pen(cfg);
  const int nrows = num_rows(pen, a2p);
  if (max_len < 1) max_len = 1;

  if (ensure(E->counters, 4 * sizeof(int32_t)) || ensure(E->retry, (size_t)n * sizeof(int32_t)))
    return WF2G_ERR_OOM_;
  int32_t* counters = (int32_t*)E->counters.p;
  if (cudaMemsetAsync(counters, 0, 4 * sizeof(int32_t), st) != cudaSuccess) return WF2G_ERR_CUDA_;

  KParams base;
  memset(&base, 0, sizeof(base));
  base.pen = pen;
  base.max_steps = cfg.max_steps;
  base.seqs = (const uint8_t*)d_seqs;
  base.p_off = d_poff;
  base.p_len = d_plen;
  base.t_off = d_toff;
  base.t_len = d_tlen;
  base.retry_items = (int32_t*)E->retry.p;
  base.retry_count = counters + 2;
  base.scores = d_scores;
  base.status = d_status;
  base.ops = (uint8_t*)d_ops;
  base.ops_off = d_opsoff;
  base.ops_len = d_opslen;
  base.max_len = max_len;
  const int table_cap = score_bound(cfg, max_len) + 1;

  // ------------------------------------------------ pass 1 (2-bit sequences)
  // Tuning knobs (environment): WF2G_RING1=0 puts the pass-1 ring in global
  // memory, WF2G_WCAP1 sets its width, WF2G_WPC1 the warps per CTA.
  const int off_bytes = (max_len < 32000) ? 2 : 4;
  PassPlan p1;
  p1.kp = base;
  p1.kp.items = nullptr;
  p1.kp.n_items = n;
  p1.kp.num_items_dev = nullptr;
  p1.kp.queue = counters + 0;
  p1.kp.final_pass = 0;
  p1.kp.ring_in_smem = env_int("WF2G_RING1", 1);
  p1.kp.wcap = next_pow2(std::min(env_int("WF2G_WCAP1", 1024), next_pow2(2 * max_len + 3)));
  p1.kp.seq_in_smem = 1;
  {
    const int nwords = ((max_len + 31) >> 5) + 2;
    size_t b = (size_t)2 * nwords * 8 + (size_t)nrows * 8;
    b = (b + 15) & ~size_t(15);
    if (p1.kp.ring_in_smem) b += (size_t)nrows * p1.kp.wcap * off_bytes;
    b = (b + 15) & ~size_t(15);
    p1.kp.smem_per_warp = (int)b;
  }
  {
    int wpc = (int)std::min<size_t>(8, E->smem_optin / std::max<size_t>(p1.kp.smem_per_warp, 1));
    wpc = env_int("WF2G_WPC1", wpc);
    p1.warps_per_cta = std::max(1, std::min(wpc, 8));
  }
  p1.smem = (size_t)p1.kp.smem_per_warp * p1.warps_per_cta;
  p1.fn = wf2g_kernel_ptr(a2p, cigar, 2, off_bytes);
  bool pass1 = p1.smem <= E->smem_optin && env_int("WF2G_PASS1", 1);
  if (pass1) {
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, p1.fn, 32 * p1.warps_per_cta, p1.smem);
    if (bps <= 0) pass1 = false;
    const int need = (n + p1.warps_per_cta - 1) / p1.warps_per_cta;
    p1.blocks = std::min(std::max(bps, 1) * E->num_sms, need);
  }
  if (pass1) {
    const int64_t warps = (int64_t)p1.blocks * p1.warps_per_cta;
    p1.kp.ring_bytes_global =
        p1.kp.ring_in_smem ? 0 : (((int64_t)nrows * p1.kp.wcap * off_bytes + 255) & ~int64_t(255));
    p1.kp.table_cap = table_cap;
    p1.kp.bits_cap = cigar ? kBits1PerWarp : 0;
    p1.kp.gscratch_per_warp =
        (p1.kp.ring_bytes_global + (cigar ? (int64_t)table_cap * 8 + kBits1PerWarp : 0) + 255) &
        ~int64_t(255);
    if (p1.kp.gscratch_per_warp > 0) {
      if (ensure(E->scratch1, (size_t)(warps * p1.kp.gscratch_per_warp))) return WF2G_ERR_OOM_;
      p1.kp.gscratch = (uint8_t*)E->scratch1.p;
    }
    int rc = launch(E, p1, st);
    if (rc) return rc;
  }

  // ------------------------------------------------ pass 2 (global ring, 8-bit)
  PassPlan p2;
  p2.kp = base;
  if (pass1) {
    p2.kp.items = (const int32_t*)E->retry.p;
    p2.kp.num_items_dev = counters + 2;
    p2.kp.n_items = 0;
  } else {
    p2.kp.items = nullptr;
    p2.kp.num_items_dev = nullptr;
    p2.kp.n_items = n;
  }
  p2.kp.queue = counters + 1;
  p2.kp.final_pass = 1;
  p2.kp.wcap = next_pow2(2 * max_len + 3);
  const int off2 = off_bytes;
  p2.kp.ring_in_smem = 0;
  const int nwords8 = ((max_len + 7) >> 3) + 2;
  const int64_t seq_bytes = (int64_t)2 * nwords8 * 8;
  p2.kp.seq_in_smem = seq_bytes <= 64 * 1024;
  {
    size_t b = (p2.kp.seq_in_smem ? (size_t)seq_bytes : 0) + (size_t)nrows * 8;
    b = (b + 15) & ~size_t(15);
    p2.kp.smem_per_warp = (int)b;
  }
  p2.warps_per_cta = kWarpsPerCta2;
  p2.smem = (size_t)p2.kp.smem_per_warp * p2.warps_per_cta;
  p2.fn = wf2g_kernel_ptr(a2p, cigar, 8, off2);
  if (p2.smem > E->smem_optin) return WF2G_ERR_ARGS_;
  {
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, p2.fn, 32 * p2.warps_per_cta, p2.smem);
    bps = std::max(1, std::min(bps, 2));
    const int need = (n + p2.warps_per_cta - 1) / p2.warps_per_cta;
    p2.blocks = std::min(bps * E->num_sms, need);
  }
  {
    int64_t warps = (int64_t)p2.blocks * p2.warps_per_cta;
    p2.kp.ring_bytes_global = ((int64_t)nrows * p2.kp.wcap * off2 + 255) & ~int64_t(255);
    p2.kp.seq_bytes_global = p2.kp.seq_in_smem ? 0 : ((seq_bytes + 255) & ~int64_t(255));
    p2.kp.table_cap = table_cap;
    int64_t fixed = p2.kp.ring_bytes_global + p2.kp.seq_bytes_global + (int64_t)table_cap * 8;
    int64_t bits = 0;
    if (cigar) {
      // every cell of every score fits: (scores) x (plen+tlen+1) diagonals
      const int64_t want = (int64_t)table_cap * (2 * (int64_t)max_len + 1) + 4 * (int64_t)max_len + 64;
      int64_t per_warp_budget = kScratch2Budget / std::max<int64_t>(warps, 1) - fixed;
      if (per_warp_budget < want && warps > E->num_sms) {
        // fewer, larger warps rather than starving each slice
        p2.blocks = std::max(1, E->num_sms / p2.warps_per_cta);
        warps = (int64_t)p2.blocks * p2.warps_per_cta;
        per_warp_budget = kScratch2Budget / warps - fixed;
      }
      bits = std::max<int64_t>(std::min(want, per_warp_budget), int64_t(1) << 20);
    }
    p2.kp.bits_cap = bits;
    p2.kp.gscratch_per_warp = (fixed + bits + 255) & ~int64_t(255);
    if (ensure(E->scratch2, (size_t)(warps * p2.kp.gscratch_per_warp))) return WF2G_ERR_OOM_;
    p2.kp.gscratch = (uint8_t*)E->scratch2.p;
  }
  return launch(E, p2, st);
}

extern "C" int wf2g_engine_align(void* engine, const wf2g_cfg_t* cfg, int n, int on_device,
                                 const char* seqs, const int64_t* p_off, const int32_t* p_len,
                                 const int64_t* t_off, const int32_t* t_len, int max_len,
                                 int32_t* scores, int32_t* status, char* ops,
                                 const int64_t* ops_off, int32_t* ops_len, void* stream) {
  Engine* E = (Engine*)engine;
  if (!E) return WF2G_ERR_NO_GPU_;
  if (n < 0 || !cfg) return WF2G_ERR_ARGS_;
  if (n == 0) return WF2G_OK_;
  if (cfg->metric != 3 && cfg->metric != 4) return WF2G_ERR_CONFIG_;
  const bool cigar = !cfg->score_only;
  if (cigar && (!ops || !ops_off || !ops_len)) return WF2G_ERR_ARGS_;
  cudaSetDevice(E->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : E->stream;

  if (on_device) {
    return plan_and_run(E, *cfg, n, seqs, p_off, p_len, t_off, t_len, max_len, scores, status,
                        ops, ops_off, ops_len, st);
  }
  // ---- host path: stage inputs, run, copy results back
  int64_t seq_end = 0, ops_end = 0;
  int mlen = 0;
  for (int i = 0; i < n; ++i) {
    if (p_len[i] < 0 || t_len[i] < 0) return WF2G_ERR_ARGS_;
    seq_end = std::max(seq_end, p_off[i] + p_len[i]);
    seq_end = std::max(seq_end, t_off[i] + t_len[i]);
    mlen = std::max(mlen, std::max(p_len[i], t_len[i]));
    if (cigar) ops_end = std::max(ops_end, ops_off[i] + (int64_t)p_len[i] + t_len[i]);
  }
  const size_t n4 = (size_t)n * 4, n8 = (size_t)n * 8;
  if (ensure(E->seqs, (size_t)seq_end + 16) || ensure(E->poff, n8) || ensure(E->plen, n4) ||
      ensure(E->toff, n8) || ensure(E->tlen, n4) || ensure(E->scores, n4) ||
      ensure(E->status, n4))
    return WF2G_ERR_OOM_;
  if (cigar && (ensure(E->ops, (size_t)ops_end + 16) || ensure(E->opsoff, n8) || ensure(E->opslen, n4)))
    return WF2G_ERR_OOM_;
  cudaError_t e = cudaSuccess;
  e = cudaMemcpyAsync(E->seqs.p, seqs, (size_t)seq_end, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(E->poff.p, p_off, n8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(E->plen.p, p_len, n4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(E->toff.p, t_off, n8, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(E->tlen.p, t_len, n4, cudaMemcpyHostToDevice, st);
  if (cigar && e == cudaSuccess) e = cudaMemcpyAsync(E->opsoff.p, ops_off, n8, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return WF2G_ERR_CUDA_;
  int rc = plan_and_run(E, *cfg, n, (const char*)E->seqs.p, (const int64_t*)E->poff.p,
                        (const int32_t*)E->plen.p, (const int64_t*)E->toff.p,
                        (const int32_t*)E->tlen.p, mlen, (int32_t*)E->scores.p,
                        (int32_t*)E->status.p, cigar ? (char*)E->ops.p : nullptr,
                        cigar ? (const int64_t*)E->opsoff.p : nullptr,
                        cigar ? (int32_t*)E->opslen.p : nullptr, st);
  if (rc) return rc;
  e = cudaMemcpyAsync(scores, E->scores.p, n4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(status, E->status.p, n4, cudaMemcpyDeviceToHost, st);
  if (cigar && e == cudaSuccess) e = cudaMemcpyAsync(ops_len, E->opslen.p, n4, cudaMemcpyDeviceToHost, st);
  if (cigar && e == cudaSuccess) e = cudaMemcpyAsync(ops, E->ops.p, (size_t)ops_end, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] CUDA error: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  return WF2G_OK_;
}

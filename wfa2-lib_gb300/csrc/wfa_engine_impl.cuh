// wfa_engine_impl.cuh -- host-side internals shared by the engine's
// translation units (wfa_engine.cu: unidirectional batches; wfa_bialign_host.cu:
// the BiWFA ultralow-memory path).  Not installed.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdlib>

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
extern "C" void* wf2g_kernel_ptr(int a2p, int cigar, int enc, int off_bytes, int heur, int wide,
                                 int ef, int lin);
extern "C" int wf2g_seq_bytes(int enc, int max_len);
extern "C" void* wf2g_bi_kernel_ptr(int a2p);
extern "C" void* wf2g_bi_pack_ptr(void);
extern "C" void* wf2g_bi_gather_ptr(void);
extern "C" size_t wf2g_bi_smem_bytes(int a2p, int scope);
extern "C" void* wf2g_pool_init_ptr(void);
extern "C" void* wf2g_fast_kernel_ptr(int cigar, int group, int width);
extern "C" void* wf2g_fast2_kernel_ptr(int cigar, int mos, int width, int d241, int wfa);

namespace eng {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

inline int ensure(DevBuf& b, size_t bytes) {
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

inline void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
}

struct BiState;  // BiWFA buffers (wfa_bialign_host.cu)
void bi_state_free(BiState* b);

// Occupancy of one kernel configuration, looked up once per engine (the
// attribute calls and the occupancy query cost more than a launch).
struct OccEntry {
  const void* fn;
  int block;
  size_t smem;
  int carve;
  int bps;
};

struct Engine {
  int device = -1;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  // host batches: a stream for the copies in, one for the copies out, and
  // an event per chunk for each (created on first use)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_in[64] = {}, ev_done[64] = {};
  int64_t launches = 0;
  // batch buffers (host-input path)
  DevBuf seqs, poff, plen, toff, tlen, scores, status, ops, opsoff, opslen, endinfo;
  // control
  DevBuf counters;  // work-queue heads and retry counts of the passes (wfa_engine.cu)
  DevBuf retry;
  DevBuf scratch0, scratch0b, scratch1, scratch2;  // fast passes, general pass 1, passes 2-4
  DevBuf pool, poolctl;  // back-trace block pool; [count, lock, ..., stack]
  BiState* bi = nullptr;
  // device-memory limits of this engine (bytes; < 0: the WF2G_SCRATCH_GB /
  // WF2G_BI_SCRATCH_GB defaults) and the cap of back-trace bytes per warp in
  // both passes (0: the first pass 1 MiB, the second sized for any alignment
  // of the batch; a pair above the cap finishes with WF_STATUS_OOM)
  int64_t scratch_budget = -1;
  int64_t bi_scratch_budget = -1;
  int64_t pool_budget = -1;  // back-trace block pool (< 0: WF2G_POOL_GB, default 32)
  int64_t bits_cap = 0;
  OccEntry occ[48];
  int n_occ = 0;
  // host batches: pinned staging of small batches, and the second engine
  // that runs every other chunk of a large batch on its own stream
  void* hstage = nullptr;
  size_t hstage_cap = 0;
  DevBuf dstage, dout;
  Engine* twin = nullptr;
};

// Blocks of `fn` per SM for `block` threads and `smem` dynamic shared memory
// (carve >= 0: the preferred shared-memory carveout, set with it).
inline int blocks_per_sm(Engine* E, const void* fn, int block, size_t smem, int carve) {
  for (int i = 0; i < E->n_occ; ++i) {
    const OccEntry& o = E->occ[i];
    if (o.fn == fn && o.block == block && o.smem == smem && o.carve == carve) return o.bps;
  }
  // the opt-in maximum, not this size: the attribute is per function and
  // process-wide, shared by every engine's launches
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem_optin);
  if (carve >= 0) cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, carve);
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, block, smem) != cudaSuccess) {
    cudaGetLastError();
    bps = 0;
  }
  if (E->n_occ < (int)(sizeof(E->occ) / sizeof(E->occ[0])))
    E->occ[E->n_occ++] = OccEntry{fn, block, smem, carve, bps};
  return bps;
}

inline int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  return (v && *v) ? atoi(v) : dflt;
}

inline Penalties make_pen(const wf2g_cfg_t& c) {
  Penalties p;
  p.match = c.match;
  p.x = c.x;
  p.o1 = c.o1;
  p.e1 = c.e1;
  if (c.metric <= 2) {
    // one component: gaps read M[s - gap_opening1] (e1 = 0, no I/D rings);
    // max_score_scope (wavefront/wavefront_components.c:47-79)
    p.x = c.metric == 0 ? 1 : c.x;  // indel has no mismatch input
    p.e1 = 0;
    p.o2 = 0;
    p.e2 = 1;
    p.R = c.metric <= 1 ? 2 : std::max(c.x, c.o1) + 1;
    p.RI1 = 1;
    p.RI2 = 1;
    return p;
  }
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

// Upper bound of the alignment score, as the reference sizes its wavefront
// table (wavefront/wavefront_components.c:101-108), for lengths <= max_len.
inline int score_bound(const wf2g_cfg_t& c, int max_len) {
  if (c.metric <= 2)  // every base a mismatch or a gap
    return (int)std::min<int64_t>((int64_t)(std::max(c.x, 0) + 2 * c.o1) * max_len + 8, INT32_MAX / 4);
  int64_t b = (int64_t)c.x * max_len + c.o1 + (int64_t)c.e1 * max_len;
  if (c.metric == 4) b = std::max<int64_t>(b, (int64_t)c.x * max_len + c.o2 + (int64_t)c.e2 * max_len);
  b += 8;
  return (int)std::min<int64_t>(b, INT32_MAX / 4);
}

// Unidirectional batch over device arrays (two passes; see wfa_engine.cu).
// d_cb/d_ce: begin/end component per pair (nullptr: M).  score_cap > 0
// replaces the score bound derived from max_len (back-trace table size).
// skip_empty: after the fast passes, wait for them and skip the general
// passes when they left no pair (small host batches, which wait anyway).
int plan_and_run(Engine* E, const wf2g_cfg_t& cfg, int n, const char* d_seqs,
                 const int64_t* d_poff, const int32_t* d_plen, const int64_t* d_toff,
                 const int32_t* d_tlen, int max_len, int32_t* d_scores, int32_t* d_status,
                 char* d_ops, const int64_t* d_opsoff, int32_t* d_opslen, const int8_t* d_cb,
                 const int8_t* d_ce, int score_cap, int32_t* d_end_info, cudaStream_t st,
                 bool skip_empty = false);

// BiWFA batch (wfa_bialign_host.cu); synchronises `st`.  end_info (may be
// null): per pair cigar->end_v, cigar->end_h and 0.
int bialign_run(Engine* E, const wf2g_cfg_t& cfg, int n, int on_device, const char* seqs,
                const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                const int32_t* t_len, int32_t* scores, int32_t* status, char* ops,
                const int64_t* ops_off, int32_t* ops_len, int32_t* end_info, cudaStream_t st);

}  // namespace eng
}  // namespace wf2g

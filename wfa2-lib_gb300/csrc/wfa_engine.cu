// wfa_engine.cu -- host side of the GB300 wavefront aligner: device buffers,
// pass planning and kernel launches behind the C interface of wfa_engine.h.
//
// A batch runs in up to four passes, all persistent kernels that pull pairs
// from a device work queue (no host round trip between them):
//   pass 1    every pair: 2-bit packed sequences, 1 MB of back-trace bytes per
//             warp; pairs with non-ACGT bytes or a longer back-trace go to a
//             retry list;
//   pass 2    the retry list, a 256-thread CTA per pair (long pairs have rows
//             of thousands of diagonals), 2-bit sequences, choice bytes in a
//             shared block pool (each pair takes blocks as its back-trace
//             grows and returns them when done), as many CTAs as the pool
//             can feed; a pair that finds the pool empty, or holds non-ACGT
//             bytes, goes to the next list;
//   pass 3    the same with 8-bit sequences and fewer CTAs;
//   pass 4    what is left, with few enough CTAs that all can hold their
//             pair's back-trace at once; a remaining overflow is reported as
//             WF_STATUS_OOM.
// Score-only runs have no back-trace: pass 2 takes the non-ACGT pairs with
// 8-bit sequences and is the last.
// Before them, in the library's headline form (gap-affine, exact, end-to-end),
// the shared-memory fast pass (wfa_fast.cu) runs over the whole batch; pass 1
// then takes only the pairs it left in its retry list.
// Each warp owns a global-memory slice holding its wavefront ring (every
// diagonal the pair can reach, so rows never wrap) and back-trace bytes; the
// slices stay L1/L2 resident.  On GB300 this measured 2x faster than a ring in
// shared memory, whose footprint capped residency at a few warps per SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <ctime>

#include "wfa_engine_impl.cuh"

namespace wf2g {
namespace eng {


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

static Engine* create_engine(int dev, int* err) {
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
          for (int h = 0; h < 2; ++h)
            for (int w = 0; w <= cig; ++w)
              for (int ef = 0; ef < 2; ++ef)
                for (int lin = 0; lin <= 1 - a2p; ++lin)
                  cudaFuncSetAttribute(wf2g_kernel_ptr(a2p, cig, enc, ob, h, w, ef, lin),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (err) *err = WF2G_OK_;
  return E;
}

extern "C" void* wf2g_engine_new(int* err) {
  const int dev = wf2g_engine_device();
  if (dev < 0) {
    if (err) *err = WF2G_ERR_NO_GPU_;
    return nullptr;
  }
  return create_engine(dev, err);
}

extern "C" void wf2g_engine_free(void* engine) {
  Engine* E = (Engine*)engine;
  if (!E) return;
  cudaSetDevice(E->device);
  DevBuf* bufs[] = {&E->seqs,   &E->poff,     &E->plen,  &E->toff,     &E->tlen,
                    &E->scores, &E->status,   &E->ops,   &E->opsoff,   &E->opslen,
                    &E->counters, &E->retry,  &E->scratch0, &E->scratch0b, &E->scratch1,
                    &E->scratch2, &E->dstage, &E->dout,
                    &E->pool,   &E->poolctl,  &E->endinfo};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (E->hstage) cudaFreeHost(E->hstage);
  bi_state_free(E->bi);
  if (E->stream) cudaStreamDestroy(E->stream);
  if (E->copy_in) cudaStreamDestroy(E->copy_in);
  if (E->copy_out) cudaStreamDestroy(E->copy_out);
  for (int c = 0; c < 64; ++c) {
    if (E->ev_in[c]) cudaEventDestroy(E->ev_in[c]);
    if (E->ev_done[c]) cudaEventDestroy(E->ev_done[c]);
  }
  if (E->twin) wf2g_engine_free(E->twin);
  delete E;
}

extern "C" int wf2g_engine_owner_device(const void* engine) {
  return engine ? ((const Engine*)engine)->device : -1;
}

extern "C" int64_t wf2g_engine_launches(const void* engine) {
  return engine ? ((const Engine*)engine)->launches : 0;
}

extern "C" int64_t wf2g_engine_bytes(const void* engine) {
  if (!engine) return 0;
  const Engine* E = (const Engine*)engine;
  const DevBuf* bufs[] = {&E->seqs,   &E->poff,     &E->plen,     &E->toff,      &E->tlen,
                          &E->scores, &E->status,   &E->ops,      &E->opsoff,    &E->opslen,
                          &E->counters, &E->retry,  &E->scratch0, &E->scratch0b, &E->scratch1,
                          &E->scratch2, &E->dstage, &E->dout,     &E->pool,      &E->poolctl,
                          &E->endinfo};
  int64_t total = (int64_t)E->hstage_cap;
  for (const DevBuf* b : bufs) total += (int64_t)b->cap;
  return total + wf2g_engine_bytes(E->twin);
}

// One persistent launch over a work list.
struct Pass {
  int enc;          // 2 or 8 bits per staged base
  int final_pass;   // 1: overflow -> WF_STATUS_OOM
  int64_t bits_cap; // back-trace bytes per warp (full CIGAR); pooled: block list + walk items
  int max_blocks_per_sm;
  int pooled;       // choice bytes in the block pool (base.pool)
  int wide;         // a 256-thread CTA per pair (pooled passes only)
};

static int run_pass(Engine* E, const wf2g_cfg_t& cfg, const KParams& base, const Pass& ps,
                    int n_upper, DevBuf& scratch, cudaStream_t st) {
  const bool a2p = (cfg.metric == 4);
  const bool cigar = !cfg.score_only;
  const int off_bytes = (base.max_len < 32000) ? 2 : 4;
  const Penalties& pen = base.pen;
  const int nrows = a2p ? pen.R + 2 * pen.RI1 + 2 * pen.RI2 : pen.R + 2 * pen.RI1;
  KParams kp = base;
  kp.final_pass = ps.final_pass;
  kp.kofs = base.max_len + 2;
  kp.row_stride = ((2 * base.max_len + 6) + 63) & ~63;
  kp.ring_bytes = (((int64_t)(nrows + 1) * kp.row_stride * off_bytes) + 255) & ~int64_t(255);
  const int64_t seq_bytes = wf2g_seq_bytes(ps.enc, base.max_len);
  kp.seq_in_smem = seq_bytes <= 48 * 1024;
  kp.seq_bytes = kp.seq_in_smem ? 0 : ((seq_bytes + 255) & ~int64_t(255));
  // staged sequences + per-row limits and initialised windows (2 x int2)
  // (+ the CTA's reduction partials and broadcast slot when a CTA is a group)
  kp.smem_per_group = (int)((((kp.seq_in_smem ? seq_bytes : 0) + (int64_t)nrows * 16 +
                              (ps.wide ? kGroupRedBytes : 0)) + 15) & ~int64_t(15));
  kp.bits_cap = cigar ? ps.bits_cap : 0;
  const int64_t table_bytes = cigar ? (int64_t)kp.table_cap * kBtRowBytes : 0;
  if (!ps.pooled) kp.pool = nullptr;
  kp.gscratch_per_group = (kp.ring_bytes + kp.seq_bytes + table_bytes + kp.bits_cap + 255) & ~int64_t(255);

  // groups per CTA: warps of one CTA (a warp per pair), or one CTA per pair
  const int tpg = ps.wide ? 256 : 32;
  int wpc = ps.wide ? 1 : (int)std::min<size_t>(8, E->smem_optin / std::max<size_t>(kp.smem_per_group, 1));
  if (!ps.wide) wpc = std::max(1, std::min(env_int("WF2G_WPC", wpc), 8));
  size_t smem = (size_t)kp.smem_per_group * wpc;
  void* fn = wf2g_kernel_ptr(a2p, cigar, ps.enc, off_bytes, base.heur, ps.wide, cfg.endsfree,
                             cfg.metric <= 2);
  if (!fn) return WF2G_ERR_CUDA_;
  // shared memory holds only the staged sequences and row limits; give the
  // rest of the SM's unified storage to L1, which caches the wavefront rows
  const int want_blocks = ps.wide ? 8 : std::max(1, 64 / wpc);
  int carve = (int)((smem * want_blocks * 100 + 228 * 1024 - 1) / (228 * 1024)) + 1;
  carve = std::max(1, std::min(carve, 100));
  int bps = blocks_per_sm(E, fn, tpg * wpc, smem, carve);
  bps = std::max(1, std::min(bps, ps.max_blocks_per_sm));
  const int need = (n_upper + wpc - 1) / wpc;
  int blocks = std::min(bps * E->num_sms, std::max(need, 1));
  if (ps.pooled) {
    // a pooled pass's warp count is a bound, not a hint: the last pass relies
    // on all of its warps holding their largest back-trace at once
    if (wpc > n_upper) {
      wpc = std::max(1, n_upper);
      smem = (size_t)kp.smem_per_group * wpc;
    }
    blocks = std::max(1, std::min(blocks, n_upper / wpc));
  }
  // bound the scratch slices by the budget
  const int64_t budget =
      E->scratch_budget >= 0 ? E->scratch_budget : (int64_t)env_int("WF2G_SCRATCH_GB", 24) << 30;
  if ((int64_t)blocks * wpc * kp.gscratch_per_group > budget)
    blocks = std::max(1, (int)(budget / (wpc * kp.gscratch_per_group)));
  if ((int64_t)wpc * kp.gscratch_per_group > budget && cigar && !ps.pooled) {
    // even one block is over the budget: shrink its back-trace slices to fit;
    // pairs whose back-trace needs more report WF_STATUS_OOM (final pass)
    const int64_t fixed = (kp.ring_bytes + kp.seq_bytes + table_bytes + 255) & ~int64_t(255);
    const int64_t bits = ((budget / wpc - fixed) & ~int64_t(255));
    if (bits < (int64_t(1) << 20)) return WF2G_ERR_OOM_;
    kp.bits_cap = bits;
    kp.gscratch_per_group = fixed + bits;
  }
  if (ensure(scratch, (size_t)blocks * wpc * kp.gscratch_per_group)) return WF2G_ERR_OOM_;
  kp.gscratch = (uint8_t*)scratch.p;
  void* args[] = {(void*)&kp};
  cudaError_t e = cudaLaunchKernel(fn, dim3(blocks), dim3(tpg * wpc), args, smem, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] kernel launch failed: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  E->launches++;
  return 0;
}

// Upper bound of the batch's sequence lengths for the fast pass: offsets stay
// int16 with room for NULL drift, and its staged sequences stay small.
constexpr int kFastMaxLen = 4096;

static int gcd_int(int a, int b) {
  while (b) {
    const int r = a % b;
    a = b;
    b = r;
  }
  return a;
}

// Whether the fast pass serves this configuration.
// wf-adaptive alone, on penalties that scale to the default's (2, 4, 1):
// the two-diagonal kernel's cut-off variant (a warp per pair)
static bool fast_wfadaptive(const wf2g_cfg_t& cfg) {
  if (cfg.heur != kHsWfadaptive || env_int("WF2G_FAST_WFA", 1) == 0 || env_int("WF2G_FAST2", 1) == 0)
    return false;
  if (cfg.x <= 0 || cfg.o1 <= 0 || cfg.e1 <= 0) return false;
  const int g = gcd_int(gcd_int(cfg.x, cfg.o1 + cfg.e1), cfg.e1);
  return cfg.x / g == 2 && (cfg.o1 + cfg.e1) / g == 4 && cfg.e1 / g == 1;
}

static bool fast_eligible(const wf2g_cfg_t& cfg, int max_len, const int8_t* d_cb,
                          const int8_t* d_ce, int score_cap) {
  return env_int("WF2G_FAST", 1) != 0 && cfg.metric == 3 &&
         (cfg.heur == 0 || fast_wfadaptive(cfg)) && !cfg.endsfree && !cfg.extension &&
         !cfg.ultralow && d_cb == nullptr && d_ce == nullptr && score_cap == 0 &&
         max_len <= kFastMaxLen && cfg.x > 0 && cfg.o1 > 0 && cfg.e1 > 0;
}

// A fast pass over pairs [0, n) (items == nullptr) or over the list `items`
// (its length at num_items_dev, at most n): one pair per CTA of G threads,
// rows of W diagonals in shared memory; pairs it leaves go to `retry` (count
// at `retry_count`).  Returns 1 when the configuration does not fit.
static int run_fast_pass(Engine* E, const wf2g_cfg_t& cfg, int G, int W, int n,
                         const int32_t* items, const int32_t* num_items_dev, const char* d_seqs,
                         const int64_t* d_poff, const int32_t* d_plen, const int64_t* d_toff,
                         const int32_t* d_tlen, int max_len, int32_t* d_scores,
                         int32_t* d_status, char* d_ops, const int64_t* d_opsoff,
                         int32_t* d_opslen, int32_t* d_end_info, int32_t* queue,
                         int32_t* retry, int32_t* retry_count, DevBuf& scratch, cudaStream_t st) {
  const bool cigar = !cfg.score_only;
  FastParams fp;
  memset(&fp, 0, sizeof(fp));
  const int g = gcd_int(gcd_int(cfg.x, cfg.o1 + cfg.e1), cfg.e1);
  fp.x = cfg.x / g;
  fp.oe = (cfg.o1 + cfg.e1) / g;
  fp.e = cfg.e1 / g;
  // a warp per pair takes two diagonals per lane when the scaled x is even
  // and the scaled e odd (wfa_fast2.cu); else one cell per thread
  const bool two = G == 32 && (fp.x & 1) == 0 && (fp.e & 1) == 1 && env_int("WF2G_FAST2", 1);
  const bool d241 = fp.x == 2 && fp.oe == 4 && fp.e == 1;
  const bool wfa = cfg.heur != 0;  // fast_eligible admits wf-adaptive alone, with d241
  if (wfa && !(two && d241)) return WF2G_ERR_CUDA_;
  void* fn = two ? wf2g_fast2_kernel_ptr(cigar, (fp.oe & 1) == 0, W, d241, wfa)
                 : wf2g_fast_kernel_ptr(cigar, G, W);
  fp.h_min_len = cfg.h_min_len;
  fp.h_max_dist = cfg.h_max_dist;
  fp.h_steps = cfg.h_steps;
  fp.probe_limit = env_int("WF2G_PROBE_LIMIT", 500);
  // (WF2G_FAST_REACH narrows the first pass, which sends more pairs to the
  // wider passes: a test of those)
  fp.reach = W / 2 - 4;
  if (W == 1024) fp.reach = std::min(fp.reach, std::max(8, env_int("WF2G_FAST_REACH", fp.reach)));
  if (!fn) return WF2G_ERR_CUDA_;
  fp.g = g;
  fp.match = cfg.match;
  // one warp per pair updates the rows in place (one slot fewer per ring)
  const int inplace = (G == 32);
  fp.R = std::max(fp.x, fp.oe) + 1 - inplace;
  fp.RI = fp.e + 1 - inplace;
  fp.max_steps = cfg.max_steps;
  fp.seqs = (const uint8_t*)d_seqs;
  fp.p_off = d_poff;
  fp.p_len = d_plen;
  fp.t_off = d_toff;
  fp.t_len = d_tlen;
  fp.items = items;
  fp.num_items_dev = num_items_dev;
  fp.n_items = n;
  fp.queue = queue;
  fp.retry_items = retry;
  fp.retry_count = retry_count;
  fp.scores = d_scores;
  fp.status = d_status;
  fp.ops = (uint8_t*)d_ops;
  fp.ops_off = d_opsoff;
  fp.ops_len = d_opslen;
  fp.end_info = d_end_info;
  fp.max_len = max_len;
  fp.nq = (max_len >> 4) + 2;
  const int nrows = fp.R + 2 * fp.RI;
  const int nw = G / 32;
  auto al16 = [](int64_t b) { return (b + 15) & ~int64_t(15); };
  int64_t off = 0;
  if (two) {
    // the two sequences' word pairs interleaved at offset 0, then the rows
    fp.q_off = 0;
    fp.rows_off = (int)al16((int64_t)2 * fp.nq * 8);
    off = al16(fp.rows_off + (int64_t)nrows * W * 2);
  } else {
    fp.rows_off = 0;
    off = al16((int64_t)nrows * W * 2);
    fp.q_off = (int)off;
    off = al16(off + (int64_t)2 * fp.nq * 8);
  }
  fp.meta_off = (int)off;
  // row limits, and (two diagonals per lane) the rows' windows
  off = al16(off + (int64_t)(nw + 1) * nrows * 8);
  fp.red_off = (int)off;
  // two step-parameter buffers, the per-warp partial reductions, a broadcast slot
  off = al16(off + 256 + (int64_t)nw * 8 * 4 + 16);
  const size_t smem = (size_t)off;
  if (smem > E->smem_optin) return 1;  // rows do not fit: the general passes take all
  fp.s_cap = W;
  fp.pair_cap = cigar && E->bits_cap > 0 ? E->bits_cap : 0;
  // per step: 4-bit choice codes (one cell per thread: 8 iterations per
  // 32-bit word; two diagonals per lane: a 16-bit entry per lane and
  // iteration of 64 words), and the row's limits (4 bytes)
  const int iters = two ? (W / 2 + 63) / 64 : (W + G - 1) / G;
  const int64_t rw = two ? (int64_t)iters * 16 : (int64_t)((iters + 7) / 8) * G;
  fp.items_off = cigar ? (int64_t)fp.s_cap * (rw * 4 + 4) : 0;
  fp.items_cap = cigar ? 4 * (int64_t)max_len + 64 : 0;
  fp.slice_bytes = cigar ? ((fp.items_off + fp.items_cap + 255) & ~int64_t(255)) : 0;
  const int bps = blocks_per_sm(E, fn, G, smem, 100);
  if (bps < 1) return 1;
  int blocks = std::min(bps * E->num_sms, std::max(n, 1));
  const int64_t budget =
      E->scratch_budget >= 0 ? E->scratch_budget : (int64_t)env_int("WF2G_SCRATCH_GB", 24) << 30;
  if (cigar && (int64_t)blocks * fp.slice_bytes > budget)
    blocks = (int)std::max<int64_t>(1, budget / fp.slice_bytes);
  if (ensure(scratch, cigar ? (size_t)blocks * fp.slice_bytes : 16)) return WF2G_ERR_OOM_;
  fp.scratch = (uint8_t*)scratch.p;
  void* args[] = {(void*)&fp};
  cudaError_t e = cudaLaunchKernel(fn, dim3(blocks), dim3(G), args, smem, st);
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] kernel launch failed: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  E->launches++;
  return 0;
}

int plan_and_run(Engine* E, const wf2g_cfg_t& cfg, int n, const char* d_seqs,
                 const int64_t* d_poff, const int32_t* d_plen, const int64_t* d_toff,
                 const int32_t* d_tlen, int max_len, int32_t* d_scores, int32_t* d_status,
                 char* d_ops, const int64_t* d_opsoff, int32_t* d_opslen, const int8_t* d_cb,
                 const int8_t* d_ce, int score_cap, int32_t* d_end_info, cudaStream_t st,
                 bool skip_empty) {
  const bool cigar = !cfg.score_only;
  if (max_len < 1) max_len = 1;
  // counters: [0..3] work queues of passes 1-4, [4..6] retry counts of passes 1-3
  // (retry lists: pass q writes list q-1, at retry + (q-1) * n), [8]/[9] work
  // queue and retry count of the first fast pass (its list at retry + 3 * n),
  // [10]/[11] those of the second (its list at retry + 4 * n), [12]/[13]
  // those of the third (its list at retry + 5 * n)
  if (ensure(E->counters, 16 * sizeof(int32_t)) || ensure(E->retry, (size_t)6 * n * sizeof(int32_t)))
    return WF2G_ERR_OOM_;
  int32_t* counters = (int32_t*)E->counters.p;
  int32_t* retry = (int32_t*)E->retry.p;
  if (cudaMemsetAsync(counters, 0, 16 * sizeof(int32_t), st) != cudaSuccess) return WF2G_ERR_CUDA_;
  bool fast = false;
  // what the fast passes leave: the list the general pass 1 takes
  const int32_t* fast_left = retry + (size_t)3 * n;
  const int32_t* fast_left_n = counters + 9;
  if (fast_eligible(cfg, max_len, d_cb, d_ce, score_cap)) {
    // the first pass: a warp per pair, rows of 1024 diagonals updated in
    // place; the second, over what the first left: rows of 2048.  A batch
    // too small to fill the GPU (the drop-in's single pair) takes four warps
    // per pair instead, which shortens each pair's steps.
    // (the wf-adaptive variant exists for a warp per pair only)
    const int small_n = cfg.heur != 0 ? 0 : env_int("WF2G_FAST_SMALL_N", 2 * E->num_sms);
    const int g1 = n <= small_n ? 128 : 32;
    int rc = run_fast_pass(E, cfg, g1, 1024, n, nullptr, nullptr, d_seqs, d_poff, d_plen, d_toff,
                           d_tlen, max_len, d_scores, d_status, d_ops, d_opsoff, d_opslen,
                           d_end_info, counters + 8, retry + (size_t)3 * n, counters + 9,
                           E->scratch0, st);
    if (rc < 0) return rc;
    fast = (rc == 0);
    if (fast && env_int("WF2G_FAST_WIDE", 1)) {
      // the pairs pass 1 left: rows of 1536 diagonals with a warp per pair
      // (10 pairs per SM; they cover every pair of the headline workload),
      // then 2048 for what remains (four warps per pair on small batches)
      const int gw = n <= small_n ? 128 : cfg.heur != 0 ? 32 : env_int("WF2G_FAST_WIDE_G", 32);
      const int g2 = gw <= 32 ? 32 : gw <= 64 ? 64 : 128;
      // (score-only wf-adaptive: 2048 at once, wfa_fast2.cu)
      const int w2 = g2 == 32 && !(cfg.heur != 0 && cfg.score_only)
                         ? env_int("WF2G_FAST_W2", 1536)
                         : 2048;
      rc = run_fast_pass(E, cfg, g2, w2 == 1536 ? 1536 : 2048, n, retry + (size_t)3 * n,
                         counters + 9, d_seqs, d_poff, d_plen, d_toff, d_tlen, max_len, d_scores,
                         d_status, d_ops, d_opsoff, d_opslen, d_end_info, counters + 10,
                         retry + (size_t)4 * n, counters + 11, E->scratch0b, st);
      if (rc < 0) return rc;
      if (rc == 0) {
        fast_left = retry + (size_t)4 * n;
        fast_left_n = counters + 11;
        if (w2 == 1536) {
          // pass 1 has finished on this stream: its scratch is free
          rc = run_fast_pass(E, cfg, 32, 2048, n, retry + (size_t)4 * n, counters + 11, d_seqs,
                             d_poff, d_plen, d_toff, d_tlen, max_len, d_scores, d_status, d_ops,
                             d_opsoff, d_opslen, d_end_info, counters + 12, retry + (size_t)5 * n,
                             counters + 13, E->scratch0, st);
          if (rc < 0) return rc;
          if (rc == 0) {
            fast_left = retry + (size_t)5 * n;
            fast_left_n = counters + 13;
          }
        }
      }
    }
    // (diagnostics: WF2G_VERBOSE=1 reads the count too, which waits for the
    // fast passes before the general ones are queued)
    const bool verbose = env_int("WF2G_VERBOSE", 0) != 0;
    if (fast && (skip_empty || verbose)) {
      // how many pairs the fast passes left (waits for them)
      int32_t left = 0;
      if (cudaMemcpyAsync(&left, fast_left_n, sizeof(left), cudaMemcpyDeviceToHost, st) !=
              cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return WF2G_ERR_CUDA_;
      if (verbose) {
        int32_t c[6] = {0, 0, 0, 0, 0, 0};  // per fast pass: pairs taken, pairs left
        if (cudaMemcpy(c, counters + 8, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess)
          return WF2G_ERR_CUDA_;
        fprintf(stderr,
                "[wfa2gpu] fast passes: %d of %d pairs left to the general kernel (left by "
                "each pass: %d %d %d)\n",
                left, n, c[1], c[3], c[5]);
      }
      if (skip_empty && left == 0) return WF2G_OK_;
    }
  }

  KParams base;
  memset(&base, 0, sizeof(base));
  base.pen = make_pen(cfg);
  base.metric = cfg.metric;
  base.max_steps = cfg.max_steps;
  base.heur = cfg.heur;
  base.h_min_len = cfg.h_min_len;
  base.h_max_dist = cfg.h_max_dist;
  base.h_steps = cfg.h_steps;
  base.h_xdrop = cfg.h_xdrop;
  base.h_zdrop = cfg.h_zdrop;
  base.h_min_k = cfg.h_min_k;
  base.h_max_k = cfg.h_max_k;
  base.pbf = cfg.pbf;
  base.pef = cfg.pef;
  base.tbf = cfg.tbf;
  base.tef = cfg.tef;
  base.extension = cfg.extension;
  base.um = cfg.um;
  base.ux = cfg.ux;
  base.uo1 = cfg.uo1;
  base.ue1 = cfg.ue1;
  base.uo2 = cfg.uo2;
  base.ue2 = cfg.ue2;
  base.end_info = d_end_info;
  base.seqs = (const uint8_t*)d_seqs;
  base.p_off = d_poff;
  base.p_len = d_plen;
  base.t_off = d_toff;
  base.t_len = d_tlen;
  base.comp_begin = d_cb;
  base.comp_end = d_ce;
  base.scores = d_scores;
  base.status = d_status;
  base.ops = (uint8_t*)d_ops;
  base.ops_off = d_opsoff;
  base.ops_len = d_opslen;
  base.max_len = max_len;
  base.table_cap = score_bound(cfg, max_len) + 1;
  if (score_cap > 0) base.table_cap = std::min(base.table_cap, score_cap + 1);

  // back-trace bytes one warp may need for any pair of the batch
  int64_t need = 0;
  if (cigar) need = (int64_t)base.table_cap * (2 * (int64_t)max_len + 1) + 4 * (int64_t)max_len + 64;
  if (cigar && E->bits_cap > 0) need = std::min(need, E->bits_cap);

  // pass 1: every pair, 2-bit sequences, 1 MB of back-trace bytes per warp;
  // pairs with non-ACGT bytes or a longer back-trace go to the next pass
  KParams k = base;
  k.items = fast ? fast_left : nullptr;
  k.num_items_dev = fast ? fast_left_n : nullptr;
  k.n_items = fast ? 0 : n;
  k.queue = counters + 0;
  k.retry_items = retry;
  k.retry_count = counters + 4;
  Pass p{2, 0, int64_t(1) << 20, 8, 0, 0};
  if (cigar) p.bits_cap = std::min(p.bits_cap, need);
  // long pairs would overflow the 1 MB slice after computing that much: they
  // go straight to the CTA-per-pair passes
  if (cigar) k.wide_min_len = env_int("WF2G_WIDE_MIN_LEN", 4096);
  int rc = run_pass(E, cfg, k, p, n, E->scratch1, st);
  if (rc) return rc;
  if (!cigar) {
    // score-only: the pairs with non-ACGT bytes, 8-bit sequences
    k = base;
    k.items = retry;
    k.num_items_dev = counters + 4;
    k.n_items = 0;
    k.queue = counters + 1;
    Pass p2{8, 1, 0, 8, 0, 0};
    return run_pass(E, cfg, k, p2, std::min(n, 8 * E->num_sms * 8), E->scratch2, st);
  }
  // passes 2-4: the overflow list, a 256-thread CTA per pair, choice bytes in
  // a shared block pool, so each pair holds what its back-trace needs, up to
  // `need` bytes (blocks of at least two of the widest rows; a row never spans
  // blocks, so a pair fills at least half of each block it holds).  Pass 2
  // (2-bit sequences) runs as many CTAs as the pool can feed at about 24 MB
  // each; pairs with non-ACGT bytes, or that find the pool empty, go to pass 3
  // (8-bit sequences, 96 MB each).  Pass 4 runs few enough CTAs that all of
  // them can hold their largest back-trace at once, so every outcome depends
  // on the pair alone; what does not fit there is reported as WF_STATUS_OOM.
  const int64_t block_bytes =
      std::max<int64_t>(int64_t(1) << 20, ((4 * (int64_t)max_len + 64) + 4095) & ~int64_t(4095));
  const int64_t pool_cap =
      E->pool_budget >= 0 ? E->pool_budget : (int64_t)env_int("WF2G_POOL_MB", 48 << 10) << 20;
  // sized for the batch: up to 64 MB per pair in flight, and at least what
  // one pair may need up to 1 GB, so a small call (the drop-in's single
  // pair) can hold a long pair's whole back-trace
  const int64_t per_pair = std::max(2 * block_bytes, std::min<int64_t>(need, int64_t(64) << 20));
  const int64_t pool_bytes = std::max(
      2 * block_bytes,
      std::min(pool_cap, std::max(std::min<int64_t>(need, int64_t(1) << 30),
                                  (int64_t)std::min(n, 8 * E->num_sms * 8) * per_pair)));
  const int nblocks = (int)std::min<int64_t>(pool_bytes / block_bytes, INT32_MAX / 2);
  if (ensure(E->pool, (size_t)nblocks * block_bytes) ||
      ensure(E->poolctl, ((size_t)nblocks + 64) * sizeof(int32_t)))
    return WF2G_ERR_OOM_;
  int32_t* ctl = (int32_t*)E->poolctl.p;
  int32_t* stack = ctl + 64;
  int32_t* count = ctl;
  int32_t* lock = ctl + 1;
  int nb = nblocks;
  void* iargs[] = {(void*)&stack, (void*)&count, (void*)&lock, (void*)&nb};
  const int igrid = std::max(1, std::min((nblocks + 255) / 256, 1024));
  if (cudaLaunchKernel(wf2g_pool_init_ptr(), dim3(igrid), dim3(256), iargs, 0, st) != cudaSuccess)
    return WF2G_ERR_CUDA_;
  E->launches++;
  const int64_t items = ((4 * (int64_t)max_len + 64) + 255) & ~int64_t(255);
  const int max_blocks =
      (int)std::min<int64_t>(nblocks, std::min<int64_t>(2 * (need / block_bytes) + 2, 16384));
  const int64_t pool_total = (int64_t)nblocks * block_bytes;
  // the back-trace bytes a pass-2 pair is expected to hold (pass 3: 4x that)
  const int64_t pair_bytes = std::max<int64_t>(1, env_int("WF2G_POOL_PAIR_MB", 24)) << 20;
  for (int q = 0; q < 3; ++q) {
    const bool final_pass = (q == 2);
    const int64_t groups = std::max<int64_t>(
        1, final_pass ? nblocks / max_blocks : pool_total / (pair_bytes << (2 * q)));
    k = base;
    k.items = retry + (size_t)q * n;
    k.num_items_dev = counters + 4 + q;
    k.n_items = 0;
    k.queue = counters + 1 + q;
    k.retry_items = final_pass ? nullptr : retry + (size_t)(q + 1) * n;
    k.retry_count = final_pass ? nullptr : counters + 5 + q;
    k.pool = (uint8_t*)E->pool.p;
    k.block_bytes = block_bytes;
    k.pool_stack = stack;
    k.pool_count = count;
    k.pool_lock = lock;
    k.max_blocks = max_blocks;
    k.pair_cap = need;
    Pass pq{q == 0 ? 2 : 8, final_pass ? 1 : 0, (int64_t)max_blocks * 4 + items, 8, 1, 1};
    rc = run_pass(E, cfg, k, pq, (int)std::min<int64_t>(n, groups), E->scratch2, st);
    if (rc) return rc;
  }
  return WF2G_OK_;
}

// ---------------------------------------------------------------- host batches
// Small batches (the per-pair drop-in wavefront_align() is one pair): every
// input goes to the GPU in one pinned staging copy and every output comes
// back in one, and the general passes are skipped when the fast passes left
// nothing.
constexpr int kSmallBatch = 64;
constexpr int64_t kSmallBytes = int64_t(4) << 20;

static int ensure_hstage(Engine* E, size_t bytes) {
  if (bytes <= E->hstage_cap) return 0;
  if (E->hstage) cudaFreeHost(E->hstage);
  E->hstage = nullptr;
  E->hstage_cap = 0;
  const size_t want = bytes + bytes / 4;
  if (cudaHostAlloc(&E->hstage, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  E->hstage_cap = want;
  return 0;
}

static size_t al16z(size_t b) { return (b + 15) & ~size_t(15); }

static double wall_s() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int host_small(Engine* E, const wf2g_cfg_t& cfg, int n, const char* seqs,
                      const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                      const int32_t* t_len, int32_t* scores, int32_t* status, char* ops,
                      const int64_t* ops_off, int32_t* ops_len, int32_t* end_info,
                      int64_t seq_end, int64_t ops_end, int mlen, cudaStream_t st) {
  const bool cigar = !cfg.score_only;
  const size_t n4 = (size_t)n * 4, n8 = (size_t)n * 8;
  // inputs: [p_off][t_off][ops_off][p_len][t_len][sequences]
  const size_t i_toff = n8, i_opsoff = 2 * n8, i_plen = 3 * n8, i_tlen = 3 * n8 + n4;
  const size_t i_seqs = al16z(3 * n8 + 2 * n4);
  const size_t in_bytes = al16z(i_seqs + (size_t)seq_end + 16);
  // outputs: [scores][status][ops_len][end_info][operations]
  const size_t o_status = n4, o_opslen = 2 * n4, o_end = 3 * n4, o_ops = al16z(6 * n4);
  const size_t out_bytes = o_ops + (cigar ? (size_t)ops_end : 0) + 16;
  if (ensure_hstage(E, in_bytes + out_bytes) || ensure(E->dstage, in_bytes) ||
      ensure(E->dout, out_bytes))
    return WF2G_ERR_OOM_;
  // diagnostics: WF2G_TIMING=2 prints the phases of every small call
  const bool timing = env_int("WF2G_TIMING", 0) >= 2;
  const double t0 = timing ? wall_s() : 0.0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (timing)
    for (auto& x : ev) cudaEventCreate(&x);
  uint8_t* const h = (uint8_t*)E->hstage;
  memcpy(h, p_off, n8);
  memcpy(h + i_toff, t_off, n8);
  if (cigar) memcpy(h + i_opsoff, ops_off, n8);
  memcpy(h + i_plen, p_len, n4);
  memcpy(h + i_tlen, t_len, n4);
  memcpy(h + i_seqs, seqs, (size_t)seq_end);
  uint8_t* const d = (uint8_t*)E->dstage.p;
  uint8_t* const q = (uint8_t*)E->dout.p;
  if (cudaMemcpyAsync(d, h, in_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return WF2G_ERR_CUDA_;
  const double t1 = timing ? wall_s() : 0.0;
  if (timing) cudaEventRecord(ev[0], st);
  const int rc = plan_and_run(
      E, cfg, n, (const char*)(d + i_seqs), (const int64_t*)d, (const int32_t*)(d + i_plen),
      (const int64_t*)(d + i_toff), (const int32_t*)(d + i_tlen), mlen, (int32_t*)q,
      (int32_t*)(q + o_status), cigar ? (char*)(q + o_ops) : nullptr,
      cigar ? (const int64_t*)(d + i_opsoff) : nullptr, cigar ? (int32_t*)(q + o_opslen) : nullptr,
      nullptr, nullptr, 0, end_info ? (int32_t*)(q + o_end) : nullptr, st, true);
  if (rc) return rc;
  if (timing) cudaEventRecord(ev[1], st);
  const double t2 = timing ? wall_s() : 0.0;
  uint8_t* const ho = h + in_bytes;
  cudaError_t e = cudaMemcpyAsync(ho, q, out_bytes - 16, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (timing) {
    float kms = 0;
    cudaEventElapsedTime(&kms, ev[0], ev[1]);
    fprintf(stderr,
            "[wfa2gpu] small call (%d pairs): staging+copy in %.1f us, plan %.1f us, "
            "copy out+wait %.1f us; kernels %.1f us\n",
            n, 1e6 * (t1 - t0), 1e6 * (t2 - t1), 1e6 * (wall_s() - t2), 1e3 * kms);
    for (auto& x : ev) cudaEventDestroy(x);
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] CUDA error: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  memcpy(scores, ho, n4);
  memcpy(status, ho + o_status, n4);
  if (end_info) memcpy(end_info, ho + o_end, 3 * n4);
  if (cigar) {
    memcpy(ops_len, ho + o_opslen, n4);
    for (int i = 0; i < n; ++i)
      if (ops_len[i] > 0) memcpy(ops + ops_off[i], ho + o_ops + ops_off[i], (size_t)ops_len[i]);
  }
  return WF2G_OK_;
}

// Large batches run in chunks of pairs on two streams (this engine's, and a
// second engine's with its own scratch), so the copies of one chunk overlap
// the kernels of the next.  Each chunk's copies move only its pairs' bytes;
// the device arrays mirror the caller's layout, so offsets stay valid.
static int host_chunked(Engine* E, const wf2g_cfg_t& cfg, int n, const char* seqs,
                        const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                        const int32_t* t_len, int32_t* scores, int32_t* status, char* ops,
                        const int64_t* ops_off, int32_t* ops_len, int32_t* end_info,
                        int64_t seq_end, int64_t ops_end, bool ops_ordered, cudaStream_t st) {
  const bool cigar = !cfg.score_only;
  const double t_start = (env_int("WF2G_VERBOSE", 0) || env_int("WF2G_TIMING", 0)) ? wall_s() : 0.0;
  const size_t n4 = (size_t)n * 4, n8 = (size_t)n * 8;
  if (ensure(E->seqs, (size_t)seq_end + 16) || ensure(E->poff, n8) || ensure(E->plen, n4) ||
      ensure(E->toff, n8) || ensure(E->tlen, n4) || ensure(E->scores, n4) ||
      ensure(E->status, n4))
    return WF2G_ERR_OOM_;
  if (cigar && (ensure(E->ops, (size_t)ops_end + 16) || ensure(E->opsoff, n8) || ensure(E->opslen, n4)))
    return WF2G_ERR_OOM_;
  if (end_info && ensure(E->endinfo, 3 * n4)) return WF2G_ERR_OOM_;
  // chunks of at least 16k pairs, at most 16; one chunk when the CIGAR regions
  // are not in pair order (the chunks' copies back could overlap)
  const int want_chunks = std::max(1, std::min(env_int("WF2G_CHUNKS", 16), 64));
  const int64_t chunk = std::max<int64_t>(16384, ((int64_t)n + want_chunks - 1) / want_chunks);
  int nchunks = (int)(((int64_t)n + chunk - 1) / chunk);
  if (cigar && !ops_ordered) nchunks = 1;
  if (nchunks > 1 && !E->twin) {
    int err = 0;
    E->twin = create_engine(E->device, &err);
    if (!E->twin) nchunks = 1;
  }
  if (E->twin) {
    E->twin->scratch_budget = E->scratch_budget;
    E->twin->pool_budget = E->pool_budget;
    E->twin->bits_cap = E->bits_cap;
  }
  const int64_t twin0 = E->twin ? E->twin->launches : 0;
  const int64_t per = ((int64_t)n + nchunks - 1) / nchunks;
  uint8_t* const dseq = (uint8_t*)E->seqs.p;
  // Copies in run back to back on their own stream, ahead of the kernels;
  // chunk c's kernels (on this engine's stream or the second engine's, in
  // turn) wait for its copies in, and its copies out (on a third stream)
  // wait for its kernels.  So neither direction of copies waits for the
  // other chunks' kernels, only for its own chunk.
  if (!E->copy_in && cudaStreamCreateWithFlags(&E->copy_in, cudaStreamNonBlocking) != cudaSuccess)
    return WF2G_ERR_CUDA_;
  if (!E->copy_out && cudaStreamCreateWithFlags(&E->copy_out, cudaStreamNonBlocking) != cudaSuccess)
    return WF2G_ERR_CUDA_;
  for (int c = 0; c < nchunks; ++c) {
    if (!E->ev_in[c] && cudaEventCreateWithFlags(&E->ev_in[c], cudaEventDisableTiming) != cudaSuccess)
      return WF2G_ERR_CUDA_;
    if (!E->ev_done[c] && cudaEventCreateWithFlags(&E->ev_done[c], cudaEventDisableTiming) != cudaSuccess)
      return WF2G_ERR_CUDA_;
  }
  // diagnostics: WF2G_TIMING=1 times the first chunk's copies in, kernels
  // and copies out (each on its own stream)
  const bool timing = env_int("WF2G_TIMING", 0) != 0;
  cudaEvent_t ev[6] = {};
  if (timing)
    for (auto& x : ev) cudaEventCreate(&x);
  // the stream the caller's batch is ordered on waits for nothing of ours
  // yet: the copies in start after what the caller queued there
  cudaEvent_t ev_start = E->ev_done[0];
  if (cudaEventRecord(ev_start, st) != cudaSuccess ||
      cudaStreamWaitEvent(E->copy_in, ev_start, 0) != cudaSuccess)
    return WF2G_ERR_CUDA_;
  int chunk_ml[64];
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < nchunks && e == cudaSuccess; ++c) {
    const int a = (int)(c * per), b = (int)std::min<int64_t>(n, (c + 1) * per);
    chunk_ml[c] = 0;
    if (a >= b) break;
    const int m = b - a;
    int64_t smin = INT64_MAX, smax = 0;
    int ml = 0;
    for (int i = a; i < b; ++i) {
      smin = std::min(smin, std::min(p_off[i], t_off[i]));
      smax = std::max(smax, std::max(p_off[i] + p_len[i], t_off[i] + t_len[i]));
      ml = std::max(ml, std::max(p_len[i], t_len[i]));
    }
    chunk_ml[c] = ml;
    if (smin > smax) smin = smax;
    const size_t m4 = (size_t)m * 4, m8 = (size_t)m * 8;
    const cudaStream_t ci = E->copy_in;
    if (timing && c == 0) cudaEventRecord(ev[0], ci);
    if (smax > smin)
      e = cudaMemcpyAsync(dseq + smin, seqs + smin, (size_t)(smax - smin), cudaMemcpyHostToDevice, ci);
    if (e == cudaSuccess) e = cudaMemcpyAsync((int64_t*)E->poff.p + a, p_off + a, m8, cudaMemcpyHostToDevice, ci);
    if (e == cudaSuccess) e = cudaMemcpyAsync((int32_t*)E->plen.p + a, p_len + a, m4, cudaMemcpyHostToDevice, ci);
    if (e == cudaSuccess) e = cudaMemcpyAsync((int64_t*)E->toff.p + a, t_off + a, m8, cudaMemcpyHostToDevice, ci);
    if (e == cudaSuccess) e = cudaMemcpyAsync((int32_t*)E->tlen.p + a, t_len + a, m4, cudaMemcpyHostToDevice, ci);
    if (cigar && e == cudaSuccess)
      e = cudaMemcpyAsync((int64_t*)E->opsoff.p + a, ops_off + a, m8, cudaMemcpyHostToDevice, ci);
    if (timing && c == 0) cudaEventRecord(ev[1], ci);
    if (e == cudaSuccess) e = cudaEventRecord(E->ev_in[c], ci);
  }
  if (e != cudaSuccess) return WF2G_ERR_CUDA_;
  for (int c = 0; c < nchunks; ++c) {
    const int a = (int)(c * per), b = (int)std::min<int64_t>(n, (c + 1) * per);
    if (a >= b) break;
    Engine* const Ec = (c & 1) ? E->twin : E;
    const cudaStream_t sc = (c & 1) ? E->twin->stream : st;
    const int m = b - a;
    const size_t m4 = (size_t)m * 4;
    if (cudaStreamWaitEvent(sc, E->ev_in[c], 0) != cudaSuccess) return WF2G_ERR_CUDA_;
    if (timing && c == 0) cudaEventRecord(ev[2], sc);
    const int rc = plan_and_run(
        Ec, cfg, m, (const char*)dseq, (const int64_t*)E->poff.p + a, (const int32_t*)E->plen.p + a,
        (const int64_t*)E->toff.p + a, (const int32_t*)E->tlen.p + a, chunk_ml[c],
        (int32_t*)E->scores.p + a, (int32_t*)E->status.p + a, cigar ? (char*)E->ops.p : nullptr,
        cigar ? (const int64_t*)E->opsoff.p + a : nullptr,
        cigar ? (int32_t*)E->opslen.p + a : nullptr, nullptr, nullptr, 0,
        end_info ? (int32_t*)E->endinfo.p + 3 * (size_t)a : nullptr, sc);
    if (rc) return rc;
    if (timing && c == 0) cudaEventRecord(ev[3], sc);
    const cudaStream_t co = E->copy_out;
    e = cudaEventRecord(E->ev_done[c], sc);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(co, E->ev_done[c], 0);
    if (timing && c == 0) cudaEventRecord(ev[4], co);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(scores + a, (int32_t*)E->scores.p + a, m4, cudaMemcpyDeviceToHost, co);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(status + a, (int32_t*)E->status.p + a, m4, cudaMemcpyDeviceToHost, co);
    if (end_info && e == cudaSuccess)
      e = cudaMemcpyAsync(end_info + 3 * (size_t)a, (int32_t*)E->endinfo.p + 3 * (size_t)a, 3 * m4,
                          cudaMemcpyDeviceToHost, co);
    if (cigar && e == cudaSuccess) {
      e = cudaMemcpyAsync(ops_len + a, (int32_t*)E->opslen.p + a, m4, cudaMemcpyDeviceToHost, co);
      // the chunk's CIGAR regions (the whole buffer when there is one chunk)
      const int64_t omin = nchunks == 1 ? 0 : ops_off[a];
      const int64_t omax =
          nchunks == 1 ? ops_end : ops_off[b - 1] + (int64_t)p_len[b - 1] + t_len[b - 1];
      if (e == cudaSuccess && omax > omin)
        e = cudaMemcpyAsync(ops + omin, (char*)E->ops.p + omin, (size_t)(omax - omin),
                            cudaMemcpyDeviceToHost, co);
    }
    if (timing && c == 0) cudaEventRecord(ev[5], co);
    if (e != cudaSuccess) return WF2G_ERR_CUDA_;
  }
  const double t_enq = (env_int("WF2G_VERBOSE", 0) || env_int("WF2G_TIMING", 0)) ? wall_s() : 0.0;
  // the copies out of the last chunk follow every chunk's kernels
  e = cudaStreamSynchronize(E->copy_out);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && nchunks > 1) e = cudaStreamSynchronize(E->twin->stream);
  if (env_int("WF2G_VERBOSE", 0) || env_int("WF2G_TIMING", 0))
    fprintf(stderr, "[wfa2gpu] host batch: %d chunks, enqueue %.1f ms, wait %.1f ms\n", nchunks,
            1e3 * (t_enq - t_start), 1e3 * (wall_s() - t_enq));
  if (E->twin) E->launches += E->twin->launches - twin0;
  if (timing) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[2], ev[3]);
    cudaEventElapsedTime(&c, ev[4], ev[5]);
    cudaPointerAttributes pa, pb;
    const int ta = cudaPointerGetAttributes(&pa, seqs) == cudaSuccess ? (int)pa.type : -1;
    const int tb = (cigar && cudaPointerGetAttributes(&pb, ops) == cudaSuccess) ? (int)pb.type : -1;
    cudaGetLastError();
    fprintf(stderr,
            "[wfa2gpu] first chunk: copies in %.1f ms, kernels %.1f ms, copies out %.1f ms "
            "(memory type of sequences %d, of operations %d)\n", a, b, c, ta, tb);
    for (auto& x : ev) cudaEventDestroy(x);
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "[wfa2gpu] CUDA error: %s\n", cudaGetErrorString(e));
    return WF2G_ERR_CUDA_;
  }
  return WF2G_OK_;
}

extern "C" int wf2g_engine_align(void* engine, const wf2g_cfg_t* cfg, int n, int on_device,
                                 const char* seqs, const int64_t* p_off, const int32_t* p_len,
                                 const int64_t* t_off, const int32_t* t_len, int max_len,
                                 int32_t* scores, int32_t* status, char* ops,
                                 const int64_t* ops_off, int32_t* ops_len, int32_t* end_info,
                                 void* stream) {
  Engine* E = (Engine*)engine;
  if (!E) return WF2G_ERR_NO_GPU_;
  if (n < 0 || !cfg) return WF2G_ERR_ARGS_;
  if (n == 0) return WF2G_OK_;
  if (cfg->metric < 0 || cfg->metric > 4) return WF2G_ERR_CONFIG_;
  const bool cigar = !cfg->score_only;
  if (cigar && (!ops || !ops_off || !ops_len)) return WF2G_ERR_ARGS_;
  cudaSetDevice(E->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : E->stream;

  if (cfg->ultralow)
    return bialign_run(E, *cfg, n, on_device, seqs, p_off, p_len, t_off, t_len, scores, status,
                       ops, ops_off, ops_len, end_info, st);
  if (on_device) {
    return plan_and_run(E, *cfg, n, seqs, p_off, p_len, t_off, t_len, max_len, scores, status,
                        ops, ops_off, ops_len, nullptr, nullptr, 0, end_info, st);
  }
  // ---- host path
  int64_t seq_end = 0, ops_end = 0;
  int mlen = 0;
  bool ops_ordered = true;  // each pair's CIGAR region after the previous one's
  for (int i = 0; i < n; ++i) {
    if (p_len[i] < 0 || t_len[i] < 0) return WF2G_ERR_ARGS_;
    seq_end = std::max(seq_end, p_off[i] + p_len[i]);
    seq_end = std::max(seq_end, t_off[i] + t_len[i]);
    mlen = std::max(mlen, std::max(p_len[i], t_len[i]));
    if (cigar) {
      ops_end = std::max(ops_end, ops_off[i] + (int64_t)p_len[i] + t_len[i]);
      if (i > 0 && ops_off[i] < ops_off[i - 1] + (int64_t)p_len[i - 1] + t_len[i - 1])
        ops_ordered = false;
    }
  }
  if (n <= kSmallBatch && seq_end <= kSmallBytes && ops_end <= kSmallBytes)
    return host_small(E, *cfg, n, seqs, p_off, p_len, t_off, t_len, scores, status, ops, ops_off,
                      ops_len, end_info, seq_end, ops_end, mlen, st);
  return host_chunked(E, *cfg, n, seqs, p_off, p_len, t_off, t_len, scores, status, ops, ops_off,
                      ops_len, end_info, seq_end, ops_end, ops_ordered, st);
}

}  // namespace eng
}  // namespace wf2g

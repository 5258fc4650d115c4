// wfa_bialign_host.cu -- host side of the BiWFA (ultralow memory) path.
//
// The reference recurses depth-first (wavefront/wavefront_bialign.c:1145-1222):
// find a breakpoint, align the left half, then the right half.  Here every
// segment of every pair at one recursion level goes to the GPU in one
// breakpoint launch (wfa_bialign.cu), the next level is built from the
// results, and all base cases run at the end in unidirectional launches with
// begin/end components.  The output equals the depth-first one: each pair's
// segments are replayed left to right, the first failure in that order ends
// the pair, and the score is the one the reference's CIGAR holds at that
// point (the level-0 breakpoint score, else the last base case's).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "wfa_bialign.cuh"
#include "wfa_engine_impl.cuh"

namespace wf2g {
namespace eng {

// wavefront/wavefront_bialign.h
constexpr int kFallbackMinScore = 250;   // WF_BIALIGN_FALLBACK_MIN_SCORE
constexpr int kFallbackMinLength = 100;  // WF_BIALIGN_FALLBACK_MIN_LENGTH
constexpr int kRecoveryMinScore = 500;   // WF_BIALIGN_RECOVERY_MIN_SCORE

struct BiState {
  DevBuf packed, pk, enc2, segs, out, rows, counter;
  DevBuf lpoff, lplen, ltoff, ltlen, lcb, lce, lscore, lstatus, lops, lopsoff, lopslen;
  DevBuf desc;
  // staging of the host-input path
  DevBuf seqs, poff, plen, toff, tlen, ops;
};

void bi_state_free(BiState* b) {
  if (!b) return;
  DevBuf* bufs[] = {&b->packed, &b->pk,      &b->enc2,   &b->segs,   &b->out,    &b->rows,
                    &b->counter, &b->lpoff,  &b->lplen,  &b->ltoff,  &b->ltlen,  &b->lcb,
                    &b->lce,    &b->lscore,  &b->lstatus, &b->lops,  &b->lopsoff, &b->lopslen,
                    &b->desc,   &b->seqs,    &b->poff,   &b->plen,   &b->toff,   &b->tlen,
                    &b->ops};
  for (DevBuf* d : bufs) release(*d);
  delete b;
}

namespace {

enum : int8_t { kPending = 0, kSplit, kBase, kTrivD, kTrivI, kFail };

struct Node {
  int32_t pair, pb, pe, tb, te;
  int32_t rem;    // score_remaining of wavefront_bialign_alignment
  int32_t child;  // kSplit: first child (the second is child+1)
  int32_t leaf;   // kBase: leaf index
  int32_t fail;   // kFail: WF_STATUS_* of the pair
  int32_t bp_score;
  int8_t cb, ce, kind;
};

#define BI_CUDA(x)                                                               \
  do {                                                                           \
    cudaError_t e_ = (x);                                                        \
    if (e_ != cudaSuccess) {                                                     \
      fprintf(stderr, "[wfa2gpu] CUDA error: %s (%s)\n", cudaGetErrorString(e_), #x); \
      return WF2G_ERR_CUDA_;                                                     \
    }                                                                            \
  } while (0)

int classic_score(const wf2g_cfg_t& c, int plen, int tlen, int s) {
  // wavefront/wavefront_compute.c:108-120
  if (c.metric <= 1) return s;  // edit and indel: the distance itself
  if (c.match == 0) return -s;
  return ((-c.match) * (plen + tlen) - s) / 2;
}

struct Ctx {
  Engine* E;
  BiState* B;
  const wf2g_cfg_t& cfg;
  cudaStream_t st;
  int n;
  const char* d_seqs;
  const int64_t* d_poff;
  const int64_t* d_toff;
  std::vector<int64_t> h_poff, h_toff;
  std::vector<int32_t> h_plen, h_tlen;
  // WF2G_BI_VERBOSE=1: per-phase wall times on stderr
  int verbose = 0;
  std::chrono::steady_clock::time_point mark;
  double ms_since_mark() {
    const auto now = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(now - mark).count();
    mark = now;
    return ms;
  }
};

// One breakpoint launch over segs; fills outs (same order).
int run_breakpoints(Ctx& C, const std::vector<BiSeg>& segs, std::vector<BiOut>& outs) {
  const int nseg = (int)segs.size();
  outs.resize(nseg);
  if (nseg == 0) return 0;
  Engine* E = C.E;
  BiState* B = C.B;
  const bool a2p = (C.cfg.metric == 4);
  const Penalties pen = make_pen(C.cfg);
  const int nc = a2p ? 5 : 3;
  const int scope = pen.R;
  int maxP = 0, maxT = 0;
  int64_t widest = 0;
  const int emin = a2p ? std::min(C.cfg.e1, C.cfg.e2) : C.cfg.e1;
  for (const BiSeg& s : segs) {
    maxP = std::max(maxP, s.pe - s.pb);
    maxT = std::max(maxT, s.te - s.tb);
  }
  (void)emin;
  widest = (int64_t)maxP + maxT + 1;
  BiParams bp;
  memset(&bp, 0, sizeof(bp));
  bp.pen = pen;
  bp.metric = C.cfg.metric;
  bp.scope = scope;
  bp.max_steps = C.cfg.max_steps;
  // the forward/reverse searches inherit the heuristic
  // (wavefront/wavefront_bialigner.c:48-56)
  bp.heur = C.cfg.heur;
  bp.h_min_len = C.cfg.h_min_len;
  bp.h_max_dist = C.cfg.h_max_dist;
  bp.h_steps = C.cfg.h_steps;
  bp.h_xdrop = C.cfg.h_xdrop;
  bp.h_min_k = C.cfg.h_min_k;
  bp.h_max_k = C.cfg.h_max_k;
  bp.seqs = (const uint8_t*)C.d_seqs;
  bp.p_off = C.d_poff;
  bp.t_off = C.d_toff;
  bp.packed = (const uint32_t*)B->packed.p;
  bp.pk_p = (const int64_t*)B->pk.p;
  bp.pk_t = (const int64_t*)B->pk.p + C.n;
  bp.enc2 = (const uint8_t*)B->enc2.p;
  bp.nseg = nseg;
  bp.kofs = maxP + 4;
  bp.stride = ((maxP + maxT + 9) + 31) & ~31;
  const int64_t nrows = 2 * (int64_t)nc * scope + 1;
  bp.rows_per_cta = nrows * bp.stride;

  // threads per segment from the widest possible wavefront of the launch
  int nt = widest <= 256 ? 64 : widest <= 2048 ? 128 : widest <= 16384 ? 256 : 512;
  nt = std::max(32, std::min(512, env_int("WF2G_BI_THREADS", nt)));
  void* fn = wf2g_bi_kernel_ptr(a2p ? 1 : 0);
  const size_t smem = wf2g_bi_smem_bytes(a2p ? 1 : 0, scope);
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, nt, smem);
  bps = std::max(1, bps);
  int ctas = std::min(nseg, bps * E->num_sms);
  const int64_t budget = E->bi_scratch_budget >= 0
                             ? E->bi_scratch_budget
                             : (int64_t)env_int("WF2G_BI_SCRATCH_GB", 32) << 30;
  const int64_t cta_bytes = bp.rows_per_cta * 4;
  if ((int64_t)ctas * cta_bytes > budget) ctas = (int)std::max<int64_t>(1, budget / cta_bytes);
  if (ensure(B->rows, (size_t)ctas * cta_bytes) || ensure(B->segs, (size_t)nseg * sizeof(BiSeg)) ||
      ensure(B->out, (size_t)nseg * sizeof(BiOut)) || ensure(B->counter, 16))
    return WF2G_ERR_OOM_;
  BI_CUDA(cudaMemcpyAsync(B->segs.p, segs.data(), (size_t)nseg * sizeof(BiSeg),
                          cudaMemcpyHostToDevice, C.st));
  BI_CUDA(cudaMemsetAsync(B->counter.p, 0, 16, C.st));
  bp.segs = (const BiSeg*)B->segs.p;
  bp.queue = (int32_t*)B->counter.p;
  bp.out = (BiOut*)B->out.p;
  bp.rows = (int32_t*)B->rows.p;
  void* args[] = {(void*)&bp};
  BI_CUDA(cudaLaunchKernel(fn, dim3(ctas), dim3(nt), args, smem, C.st));
  E->launches++;
  BI_CUDA(cudaMemcpyAsync(outs.data(), B->out.p, (size_t)nseg * sizeof(BiOut),
                          cudaMemcpyDeviceToHost, C.st));
  BI_CUDA(cudaStreamSynchronize(C.st));
  if (C.verbose)
    fprintf(stderr, "[wfa2gpu] breakpoints: %d segments (max %d x %d), %d CTAs x %d threads, %.3f ms\n",
            nseg, maxP, maxT, ctas, nt, C.ms_since_mark());
  return 0;
}

// Breakpoint launch over node ids (longest segments first).
int search_nodes(Ctx& C, std::vector<Node>& nodes, std::vector<int>& ids,
                 std::vector<BiOut>& outs) {
  std::sort(ids.begin(), ids.end(), [&](int a, int b) {
    const int64_t la = (int64_t)nodes[a].pe - nodes[a].pb + nodes[a].te - nodes[a].tb;
    const int64_t lb = (int64_t)nodes[b].pe - nodes[b].pb + nodes[b].te - nodes[b].tb;
    return la != lb ? la > lb : a < b;
  });
  std::vector<BiSeg> segs(ids.size());
  for (size_t i = 0; i < ids.size(); ++i) {
    const Node& nd = nodes[ids[i]];
    segs[i] = BiSeg{nd.pair, nd.pb, nd.pe, nd.tb, nd.te, nd.cb, nd.ce, 0};
  }
  return run_breakpoints(C, segs, outs);
}

}  // namespace

int bialign_run(Engine* E, const wf2g_cfg_t& cfg, int n, int on_device, const char* seqs,
                const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                const int32_t* t_len, int32_t* scores, int32_t* status, char* ops,
                const int64_t* ops_off, int32_t* ops_len, int32_t* end_info, cudaStream_t st) {
  if (!E->bi) {
    E->bi = new (std::nothrow) BiState();
    if (!E->bi) return WF2G_ERR_OOM_;
  }
  BiState* B = E->bi;
  const bool cigar = !cfg.score_only;
  Ctx C{E, B, cfg, st, n, nullptr, nullptr, nullptr, {}, {}, {}, {}, 0, {}};
  C.verbose = env_int("WF2G_BI_VERBOSE", 0);
  C.mark = std::chrono::steady_clock::now();
  C.h_poff.resize(n);
  C.h_toff.resize(n);
  C.h_plen.resize(n);
  C.h_tlen.resize(n);
  std::vector<int64_t> h_opsoff;
  const int32_t* d_plen = nullptr;
  const int32_t* d_tlen = nullptr;
  const size_t n4 = (size_t)n * 4, n8 = (size_t)n * 8;

  // ---- inputs on the device, lengths and offsets on the host
  if (on_device) {
    C.d_seqs = seqs;
    C.d_poff = p_off;
    C.d_toff = t_off;
    d_plen = p_len;
    d_tlen = t_len;
    BI_CUDA(cudaMemcpyAsync(C.h_poff.data(), p_off, n8, cudaMemcpyDeviceToHost, st));
    BI_CUDA(cudaMemcpyAsync(C.h_toff.data(), t_off, n8, cudaMemcpyDeviceToHost, st));
    BI_CUDA(cudaMemcpyAsync(C.h_plen.data(), p_len, n4, cudaMemcpyDeviceToHost, st));
    BI_CUDA(cudaMemcpyAsync(C.h_tlen.data(), t_len, n4, cudaMemcpyDeviceToHost, st));
    if (cigar) {
      h_opsoff.resize(n);
      BI_CUDA(cudaMemcpyAsync(h_opsoff.data(), ops_off, n8, cudaMemcpyDeviceToHost, st));
    }
    BI_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i)
      if (C.h_plen[i] < 0 || C.h_tlen[i] < 0) return WF2G_ERR_ARGS_;
  } else {
    int64_t seq_end = 0;
    for (int i = 0; i < n; ++i) {
      if (p_len[i] < 0 || t_len[i] < 0) return WF2G_ERR_ARGS_;
      seq_end = std::max(seq_end, std::max(p_off[i] + p_len[i], t_off[i] + t_len[i]));
    }
    memcpy(C.h_poff.data(), p_off, n8);
    memcpy(C.h_toff.data(), t_off, n8);
    memcpy(C.h_plen.data(), p_len, n4);
    memcpy(C.h_tlen.data(), t_len, n4);
    if (cigar) h_opsoff.assign(ops_off, ops_off + n);
    if (ensure(B->seqs, (size_t)seq_end + 16) || ensure(B->poff, n8) || ensure(B->toff, n8) ||
        ensure(B->plen, n4) || ensure(B->tlen, n4))
      return WF2G_ERR_OOM_;
    BI_CUDA(cudaMemcpyAsync(B->seqs.p, seqs, (size_t)seq_end, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaMemcpyAsync(B->poff.p, p_off, n8, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaMemcpyAsync(B->toff.p, t_off, n8, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaMemcpyAsync(B->plen.p, p_len, n4, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaMemcpyAsync(B->tlen.p, t_len, n4, cudaMemcpyHostToDevice, st));
    C.d_seqs = (const char*)B->seqs.p;
    C.d_poff = (const int64_t*)B->poff.p;
    C.d_toff = (const int64_t*)B->toff.p;
    d_plen = (const int32_t*)B->plen.p;
    d_tlen = (const int32_t*)B->tlen.p;
  }

  // ---- 2-bit packing for the breakpoint search
  {
    std::vector<int64_t> pk(2 * (size_t)n);
    int64_t words = 0;
    for (int i = 0; i < n; ++i) {
      pk[i] = words;
      words += packed_words(C.h_plen[i]);
      pk[n + i] = words;
      words += packed_words(C.h_tlen[i]);
    }
    if (ensure(B->packed, (size_t)words * 4 + 16) || ensure(B->pk, 2 * n8) || ensure(B->enc2, n))
      return WF2G_ERR_OOM_;
    BI_CUDA(cudaMemcpyAsync(B->pk.p, pk.data(), 2 * n8, cudaMemcpyHostToDevice, st));
    PackParams q;
    q.seqs = (const uint8_t*)C.d_seqs;
    q.p_off = C.d_poff;
    q.p_len = d_plen;
    q.t_off = C.d_toff;
    q.t_len = d_tlen;
    q.packed = (uint32_t*)B->packed.p;
    q.pk_p = (const int64_t*)B->pk.p;
    q.pk_t = (const int64_t*)B->pk.p + n;
    q.enc2 = (uint8_t*)B->enc2.p;
    q.n = n;
    void* args[] = {(void*)&q};
    const int grid = std::max(1, std::min(n, E->num_sms * 8));
    BI_CUDA(cudaLaunchKernel(wf2g_bi_pack_ptr(), dim3(grid), dim3(256), args, 0, st));
    E->launches++;
  }

  std::vector<int32_t> r_score(n), r_status(n), r_len(n, 0);
  // cigar->end_v/end_h: the sequence lengths when the score-only search
  // completes (wavefront/wavefront_bialign.c:1248-1257), or when a full
  // alignment's top level splits at a breakpoint (:1214-1220); a top level
  // that went to the base case keeps the cleared end (:159-194)
  std::vector<int32_t> r_end((size_t)3 * n, -1);
  if (C.verbose) {
    BI_CUDA(cudaStreamSynchronize(st));
    fprintf(stderr, "[wfa2gpu] BiWFA inputs + packing: %.3f ms\n", C.ms_since_mark());
  }

  // ---- score only (wavefront/wavefront_bialign.c:1226-1263)
  if (!cigar) {
    std::vector<Node> nodes(n);
    std::vector<int> ids(n);
    for (int i = 0; i < n; ++i) {
      nodes[i] = Node{i, 0, C.h_plen[i], 0, C.h_tlen[i], INT_MAX, -1, -1, 0, 0, 0, 0, kPending};
      ids[i] = i;
    }
    std::vector<BiOut> outs;
    int rc = search_nodes(C, nodes, ids, outs);
    if (rc) return rc;
    for (size_t j = 0; j < ids.size(); ++j) {
      const int i = ids[j];
      const BiOut& o = outs[j];
      if (o.status == kBiOk || o.status == kBiEndReached) {
        r_score[i] = classic_score(cfg, C.h_plen[i], C.h_tlen[i],
                                   o.status == kBiOk ? o.score : o.reached);
        r_status[i] = kStCompleted;
        r_end[3 * (size_t)i] = C.h_plen[i];
        r_end[3 * (size_t)i + 1] = C.h_tlen[i];
      } else {
        r_score[i] = INT32_MIN;  // cigar_clear()
        r_status[i] = o.status == kBiMaxSteps ? kStMaxSteps : kStUnattainable;
      }
    }
  } else {
    // ---- full alignment: recursion level by level
    std::vector<Node> nodes;
    nodes.reserve((size_t)n * 4);
    std::vector<int> frontier(n);
    for (int i = 0; i < n; ++i) {
      const int mx = std::max(C.h_plen[i], C.h_tlen[i]);
      // wavefront/wavefront_bialign.c:1276-1281
      nodes.push_back(Node{i, 0, C.h_plen[i], 0, C.h_tlen[i],
                           mx <= kFallbackMinLength ? 0 : INT_MAX, -1, -1, 0, 0, 0, 0, kPending});
      frontier[i] = i;
    }
    std::vector<int> base_nodes;
    while (!frontier.empty()) {
      std::vector<int> search;
      for (int id : frontier) {
        Node& nd = nodes[id];
        const int pl = nd.pe - nd.pb, tl = nd.te - nd.tb;
        if (tl == 0) nd.kind = kTrivD;
        else if (pl == 0) nd.kind = kTrivI;
        else if (nd.rem <= kFallbackMinScore) {
          nd.kind = kBase;
          base_nodes.push_back(id);
        } else {
          search.push_back(id);
        }
      }
      std::vector<int> next;
      if (!search.empty()) {
        std::vector<BiOut> outs;
        int rc = search_nodes(C, nodes, search, outs);
        if (rc) return rc;
        for (size_t j = 0; j < search.size(); ++j) {
          const int id = search[j];
          const BiOut& o = outs[j];
          if (o.status == kBiOk) {
            const int bh = o.off_f, bv = o.off_f - o.k_f;
            const Node cur = nodes[id];
            const int c0 = (int)nodes.size();
            nodes[id].kind = kSplit;
            nodes[id].child = c0;
            nodes[id].bp_score = o.score;
            nodes.push_back(Node{cur.pair, cur.pb, cur.pb + bv, cur.tb, cur.tb + bh, o.score_f, -1,
                                 -1, 0, 0, cur.cb, (int8_t)o.comp, kPending});
            nodes.push_back(Node{cur.pair, cur.pb + bv, cur.pe, cur.tb + bh, cur.te, o.score_r,
                                 -1, -1, 0, 0, (int8_t)o.comp, cur.ce, kPending});
            next.push_back(c0);
            next.push_back(c0 + 1);
          } else if (o.status == kBiEndReached && o.reached <= kRecoveryMinScore) {
            // wavefront/wavefront_bialign.c:1084-1114
            nodes[id].kind = kBase;
            base_nodes.push_back(id);
          } else {
            nodes[id].kind = kFail;
            nodes[id].fail = o.status == kBiMaxSteps ? kStMaxSteps : kStUnattainable;
          }
        }
      }
      frontier.swap(next);
    }

    // ---- base cases: unidirectional launches, bucketed by sequence length
    const int nl = (int)base_nodes.size();
    std::vector<int> order(base_nodes);
    auto mlen = [&](int id) { return std::max(nodes[id].pe - nodes[id].pb, nodes[id].te - nodes[id].tb); };
    std::sort(order.begin(), order.end(), [&](int a, int b) { return mlen(a) < mlen(b); });
    std::vector<int64_t> lpoff(nl), ltoff(nl), lopsoff(nl + 1, 0);
    std::vector<int32_t> lplen(nl), ltlen(nl);
    std::vector<int8_t> lcb(nl), lce(nl);
    for (int j = 0; j < nl; ++j) {
      Node& nd = nodes[order[j]];
      nd.leaf = j;
      lpoff[j] = C.h_poff[nd.pair] + nd.pb;
      ltoff[j] = C.h_toff[nd.pair] + nd.tb;
      lplen[j] = nd.pe - nd.pb;
      ltlen[j] = nd.te - nd.tb;
      lcb[j] = nd.cb;
      lce[j] = nd.ce;
      lopsoff[j + 1] = lopsoff[j] + lplen[j] + ltlen[j];
    }
    std::vector<int32_t> lscore(nl), lstatus(nl), lopslen(nl);
    if (nl > 0) {
      const size_t l4 = (size_t)nl * 4, l8 = (size_t)nl * 8;
      if (ensure(B->lpoff, l8) || ensure(B->ltoff, l8) || ensure(B->lplen, l4) ||
          ensure(B->ltlen, l4) || ensure(B->lcb, nl) || ensure(B->lce, nl) ||
          ensure(B->lscore, l4) || ensure(B->lstatus, l4) || ensure(B->lopslen, l4) ||
          ensure(B->lopsoff, l8) || ensure(B->lops, (size_t)lopsoff[nl] + 16))
        return WF2G_ERR_OOM_;
      BI_CUDA(cudaMemcpyAsync(B->lpoff.p, lpoff.data(), l8, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->ltoff.p, ltoff.data(), l8, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->lplen.p, lplen.data(), l4, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->ltlen.p, ltlen.data(), l4, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->lcb.p, lcb.data(), nl, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->lce.p, lce.data(), nl, cudaMemcpyHostToDevice, st));
      BI_CUDA(cudaMemcpyAsync(B->lopsoff.p, lopsoff.data(), l8, cudaMemcpyHostToDevice, st));
      // base cases score at most max(250, 500 on recovery), or a whole pair
      // of length <= 100 (wavefront/wavefront_bialign.c:1160-1164,1105-1107)
      const int cap = std::max(score_bound(cfg, kFallbackMinLength), kRecoveryMinScore + 64);
      const int bounds[3] = {1024, 30000, INT_MAX};
      // the base aligner runs without heuristic (wavefront/wavefront_bialigner.c:64-66)
      wf2g_cfg_t bcfg = cfg;
      bcfg.heur = 0;
      int j0 = 0;
      for (int b = 0; b < 3 && j0 < nl; ++b) {
        int j1 = j0;
        while (j1 < nl && std::max(lplen[j1], ltlen[j1]) <= bounds[b]) ++j1;
        if (j1 == j0) continue;
        const int ml = std::max(lplen[j1 - 1], ltlen[j1 - 1]);
        int rc = plan_and_run(E, bcfg, j1 - j0, C.d_seqs, (const int64_t*)B->lpoff.p + j0,
                              (const int32_t*)B->lplen.p + j0, (const int64_t*)B->ltoff.p + j0,
                              (const int32_t*)B->ltlen.p + j0, ml,
                              (int32_t*)B->lscore.p + j0, (int32_t*)B->lstatus.p + j0,
                              (char*)B->lops.p, (const int64_t*)B->lopsoff.p + j0,
                              (int32_t*)B->lopslen.p + j0, (const int8_t*)B->lcb.p + j0,
                              (const int8_t*)B->lce.p + j0, cap, nullptr, st);
        if (rc) return rc;
        j0 = j1;
      }
      BI_CUDA(cudaMemcpyAsync(lscore.data(), B->lscore.p, l4, cudaMemcpyDeviceToHost, st));
      BI_CUDA(cudaMemcpyAsync(lstatus.data(), B->lstatus.p, l4, cudaMemcpyDeviceToHost, st));
      BI_CUDA(cudaMemcpyAsync(lopslen.data(), B->lopslen.p, l4, cudaMemcpyDeviceToHost, st));
      BI_CUDA(cudaStreamSynchronize(st));
      if (C.verbose) fprintf(stderr, "[wfa2gpu] base cases: %d, %.3f ms\n", nl, C.ms_since_mark());
    }

    // ---- depth-first replay per pair: pieces, score, status
    std::vector<CopyDesc> desc;
    std::vector<int> stack;
    for (int i = 0; i < n; ++i) {
      int32_t last_score = INT32_MIN;  // cigar_resize() clears the score
      int fail = 0;
      int64_t len = 0;
      const size_t d0 = desc.size();
      stack.assign(1, i);
      while (!stack.empty() && !fail) {
        const Node& nd = nodes[stack.back()];
        stack.pop_back();
        const int pl = nd.pe - nd.pb, tl = nd.te - nd.tb;
        switch (nd.kind) {
          case kSplit:
            stack.push_back(nd.child + 1);
            stack.push_back(nd.child);
            break;
          case kTrivD:
          case kTrivI: {
            const int m = nd.kind == kTrivD ? pl : tl;
            if (m > 0) desc.push_back(CopyDesc{0, h_opsoff[i] + len, m, nd.kind == kTrivD ? 'D' : 'I'});
            len += m;
            break;
          }
          case kBase: {
            const int j = nd.leaf;
            // wavefront/wavefront_bialign.c:180-193: the base CIGAR's score is
            // copied, then anything but ALG_COMPLETED fails the pair
            last_score = lscore[j];
            if (lstatus[j] == kStCompleted) {
              if (lopslen[j] > 0) desc.push_back(CopyDesc{lopsoff[j], h_opsoff[i] + len, lopslen[j], 0});
              len += lopslen[j];
            } else {
              fail = lstatus[j] == kStOOM ? kStOOM : kStUnattainable;
            }
            break;
          }
          case kFail:
            fail = nd.fail;
            break;
          default:
            fail = kStUnattainable;
            break;
        }
      }
      if (fail) {
        desc.resize(d0);
        r_status[i] = fail;
        r_score[i] = last_score;
        r_len[i] = 0;
      } else {
        r_status[i] = kStCompleted;
        r_score[i] = nodes[i].kind == kSplit
                         ? classic_score(cfg, C.h_plen[i], C.h_tlen[i], nodes[i].bp_score)
                         : last_score;
        r_len[i] = (int32_t)len;
        if (nodes[i].kind == kSplit) {
          r_end[3 * (size_t)i] = C.h_plen[i];
          r_end[3 * (size_t)i + 1] = C.h_tlen[i];
        }
      }
    }

    // ---- CIGAR assembly on the device
    char* d_out_ops = ops;
    int64_t ops_end = 0;
    if (!on_device) {
      for (int i = 0; i < n; ++i)
        ops_end = std::max(ops_end, h_opsoff[i] + (int64_t)C.h_plen[i] + C.h_tlen[i]);
      if (ensure(B->ops, (size_t)ops_end + 16)) return WF2G_ERR_OOM_;
      d_out_ops = (char*)B->ops.p;
    }
    if (!desc.empty()) {
      if (ensure(B->desc, desc.size() * sizeof(CopyDesc))) return WF2G_ERR_OOM_;
      BI_CUDA(cudaMemcpyAsync(B->desc.p, desc.data(), desc.size() * sizeof(CopyDesc),
                              cudaMemcpyHostToDevice, st));
      const CopyDesc* dd = (const CopyDesc*)B->desc.p;
      int nd = (int)desc.size();
      const uint8_t* src = (const uint8_t*)B->lops.p;
      uint8_t* dst = (uint8_t*)d_out_ops;
      void* args[] = {(void*)&dd, (void*)&nd, (void*)&src, (void*)&dst};
      const int grid = std::max(1, std::min((nd + 7) / 8, E->num_sms * 16));
      BI_CUDA(cudaLaunchKernel(wf2g_bi_gather_ptr(), dim3(grid), dim3(256), args, 0, st));
      E->launches++;
    }
    if (!on_device) {
      BI_CUDA(cudaMemcpyAsync(ops, d_out_ops, (size_t)ops_end, cudaMemcpyDeviceToHost, st));
    }
  }

  // ---- per-pair results
  if (C.verbose) {
    BI_CUDA(cudaStreamSynchronize(st));
    fprintf(stderr, "[wfa2gpu] assembly: %.3f ms\n", C.ms_since_mark());
  }
  for (int i = 0; i < n; ++i) r_end[3 * (size_t)i + 2] = 0;
  if (on_device) {
    BI_CUDA(cudaMemcpyAsync(scores, r_score.data(), n4, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaMemcpyAsync(status, r_status.data(), n4, cudaMemcpyHostToDevice, st));
    if (cigar) BI_CUDA(cudaMemcpyAsync(ops_len, r_len.data(), n4, cudaMemcpyHostToDevice, st));
    if (end_info)
      BI_CUDA(cudaMemcpyAsync(end_info, r_end.data(), 3 * n4, cudaMemcpyHostToDevice, st));
    BI_CUDA(cudaStreamSynchronize(st));
  } else {
    BI_CUDA(cudaStreamSynchronize(st));
    memcpy(scores, r_score.data(), n4);
    memcpy(status, r_status.data(), n4);
    if (cigar) memcpy(ops_len, r_len.data(), n4);
    if (end_info) memcpy(end_info, r_end.data(), 3 * n4);
  }
  return WF2G_OK_;
}

}  // namespace eng
}  // namespace wf2g

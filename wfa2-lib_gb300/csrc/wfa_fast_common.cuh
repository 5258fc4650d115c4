// wfa_fast_common.cuh -- pieces shared by the two shared-memory fast kernels
// (wfa_fast.cu: one cell per thread; wfa_fast2.cu: two diagonals per lane):
// sequence staging, the 16-base LCP, and the back-trace walk with its
// forward replay.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "wfa_kernels.cuh"

namespace wf2g {

// Longest common prefix of P[v..] and T[h..], at most lim bases (lim >= 0,
// v+lim <= plen, h+lim <= tlen): 16-base windows, XOR + count leading zeros
// (wavefront/wavefront_extend_kernels.c:68-92).  Q[i*S] = {word i+1, word i}
// (S = 2: the two sequences' word pairs interleaved).
template <int S = 1>
__device__ __forceinline__ int fast_lcp(const uint2* __restrict__ QP, const uint2* __restrict__ QT,
                                        int v, int h, int lim) {
  int L = 0;
  while (L < lim) {
    const int pv = v + L, ph = h + L;
    const uint2 a = QP[(pv >> 4) * S];
    const uint2 b = QT[(ph >> 4) * S];
    const uint32_t d = __funnelshift_l(a.x, a.y, (uint32_t)pv << 1) ^
                       __funnelshift_l(b.x, b.y, (uint32_t)ph << 1);
    if (d) {
      L += __clz(d) >> 1;
      break;
    }
    L += 16;
  }
  return L < lim ? L : lim;
}

template <int G>
__device__ __forceinline__ void fast_sync() {
  if (G == 32) __syncwarp();
  else __syncthreads();
}

// Stages one sequence as word pairs: base i at bits [31-2(i%16), 30-2(i%16)]
// of word i/16, Q[i*S] = {word i+1, word i} for i < nq (words past the
// sequence are 0).  Returns false (group-uniform) if a byte is not A/C/G/T.
template <int G, int S = 1>
__device__ bool fast_stage(const uint8_t* __restrict__ src, int len, uint2* Q, int nq, int t) {
  const int lane = t & 31;
  bool ok = true;
  // 32 bases per warp pass -> words 2b and 2b+1; words up to index nq are needed
  const int nblk = (nq >> 1) + 1;
  for (int b = t >> 5; b < nblk; b += G / 32) {
    const int i = (b << 5) + lane;
    uint32_t code = 0;
    if (i < len) {
      const uint8_t c = src[i];
      ok &= (c == 'A') | (c == 'C') | (c == 'G') | (c == 'T');
      code = (c >> 1) & 3u;  // A0 C1 T2 G3: a bijection on ACGT
    }
    const int sh = 30 - 2 * (lane & 15);
    const uint32_t w0 = __reduce_or_sync(kFull, lane < 16 ? code << sh : 0u);
    const uint32_t w1 = __reduce_or_sync(kFull, lane >= 16 ? code << sh : 0u);
    const int i0 = 2 * b, i1 = 2 * b + 1;
    // word j goes to Q[j].y and Q[j-1].x
    if (lane == 0) {
      if (i0 < nq) Q[i0 * S].y = w0;
      if (i0 >= 1 && i0 - 1 < nq) Q[(i0 - 1) * S].x = w0;
    } else if (lane == 1) {
      if (i1 < nq) Q[i1 * S].y = w1;
      if (i1 - 1 < nq) Q[(i1 - 1) * S].x = w1;
    }
  }
  if (G == 32) return __all_sync(kFull, ok);
  return __syncthreads_and(ok);
}

// The back-trace of one pair by one warp (every lane calls it alike), from
// (s, k_end) in M to (0, 0), then the forward replay into the pair's CIGAR
// (wavefront/wavefront_backtrace.c:320-529).  code_at(ss, kk, bad) returns
// the choice code of cell (ss, kk): bits 0-1 the source of M (0 mismatch,
// 1 deletion, 2 insertion), bit 2 "insertion extended", bit 3 "deletion
// extended"; it sets bad for a cell outside its row.  The walk records the
// operations backwards in items (an 'E' at every M visit); the replay
// re-extends each M visit with the same LCP (staged word pairs at stride
// QS).  Writes the pair's score, status, CIGAR length and end position;
// returns false if the trace was inconsistent or did not fit (the caller
// leaves the pair to the general kernel).
template <int QS, typename CodeAt>
__device__ bool fast_backtrace(const FastParams& p, int pair, int plen, int tlen, int s,
                               int k_end, int score, int S, const uint2* QP, const uint2* QT,
                               uint8_t* items, int lane, CodeAt code_at) {
  bool bad = false;
  int64_t n = 0;
  auto emit = [&](uint8_t op) -> bool {
    if (n + 1 > p.items_cap) return false;
    if (lane == 0) items[n] = op;
    ++n;
    return true;
  };
  // One cell of the walk: (ss, kk) entered in state st (0 M, 1 D, 2 I)
  // with its code c.  Emits its operations and moves to the next cell,
  // which is successor l of this one: 1 mismatch (ss-x, kk), 2 deletion
  // extended (ss-e, kk+1), 3 deletion opened (ss-(o+e), kk+1), 4
  // insertion extended (ss-e, kk-1), 5 insertion opened (ss-(o+e),
  // kk-1).  Returns 0 (moved), 1 (reached score 0) or -1 (inconsistent).
  auto resolve = [&](int& ss, int& kk, int& st, uint32_t c, bool cbad, int& l) -> int {
    if (st == 0) {
      if (!emit('E')) return -1;
      if (ss == 0) return kk == 0 ? 1 : -1;
      if (cbad) return -1;
      const uint32_t src = c & 3u;
      if (src == 0) {
        if (!emit('X')) return -1;
        ss -= p.x;
        l = 1;
        return ss >= 0 ? 0 : -1;
      }
      st = (src == 1) ? 1 : 2;  // a gap chain starts in this cell
    } else if (cbad) {
      return -1;
    }
    // a gap cell: deletions move to k+1, insertions to k-1; the extend
    // bit says whether the gap continues (score - e) or was opened from
    // M (score - (o+e))
    const bool del = (st == 1);
    if (!emit(del ? 'D' : 'I')) return -1;
    kk += del ? 1 : -1;
    if (c & (del ? 8u : 4u)) {
      ss -= p.e;
      l = del ? 2 : 4;
      return ss > 0 ? 0 : -1;  // a gap cannot begin the alignment
    }
    ss -= p.oe;
    st = 0;
    l = del ? 3 : 5;
    return ss >= 0 ? 0 : -1;
  };
  // Walk from (s, k_end) in M to (0, 0), two cells per round trip to
  // memory: knowing the code of the cell being left, lanes 0-5 load the
  // code of the next cell and of the five cells reachable from it;
  // resolving the next cell then finds its successor's code loaded.
  int ss = s, kk = k_end, st = 0;
  bool cbad = false;
  uint32_t c = ss > 0 ? code_at(ss, kk, cbad) : 0u;
  while (true) {
    int l = 0;
    int r = resolve(ss, kk, st, c, cbad, l);
    if (r != 0) {
      bad = (r < 0);
      break;
    }
    // the cell entered, (ss, kk), and its successors
    int qs = ss, qk = kk;
    if (lane == 1) { qs = ss - p.x; }
    else if (lane == 2) { qs = ss - p.e; qk = kk + 1; }
    else if (lane == 3) { qs = ss - p.oe; qk = kk + 1; }
    else if (lane == 4) { qs = ss - p.e; qk = kk - 1; }
    else if (lane == 5) { qs = ss - p.oe; qk = kk - 1; }
    bool qbad = false;
    uint32_t qc = 0u;
    if (lane < 6 && qs > 0) qc = code_at(qs, qk, qbad);
    c = __shfl_sync(kFull, qc, 0);
    cbad = __shfl_sync(kFull, (int)qbad, 0) != 0;
    r = resolve(ss, kk, st, c, cbad, l);
    if (r != 0) {
      bad = (r < 0);
      break;
    }
    c = __shfl_sync(kFull, qc, l);
    cbad = __shfl_sync(kFull, (int)qbad, l) != 0;
  }
  __syncwarp();
  // forward replay
  int out_n = 0, v = 0, h = 0;
  uint8_t* const out = p.ops + p.ops_off[pair];
  const int cap = plen + tlen;
  for (int64_t base = n - 1; base >= 0 && !bad; base -= 32) {
    const uint32_t mine = (base - lane >= 0) ? items[base - lane] : 0u;
    const int cnt = base + 1 < 32 ? (int)base + 1 : 32;
    for (int q = 0; q < cnt; ++q) {
      const uint32_t it = __shfl_sync(kFull, mine, q);
      if (it == 'E') {
        const int L = fast_lcp<QS>(QP, QT, v, h, min(plen - v, tlen - h));
        if (out_n + L > cap) { bad = true; break; }
        for (int u = lane; u < L; u += 32) out[out_n + u] = 'M';
        out_n += L;
        v += L;
        h += L;
      } else {
        if (it == 'X') { bad = (v >= plen) || (h >= tlen); ++v; ++h; }
        else if (it == 'I') { bad = h >= tlen; ++h; }
        else { bad = v >= plen; ++v; }
        if (bad || out_n >= cap) { bad = true; break; }
        if (lane == 0) out[out_n] = (uint8_t)it;
        ++out_n;
      }
    }
  }
  if (v != plen || h != tlen) bad = true;
  if (lane == 0 && !bad) {
    p.scores[pair] = score;
    p.status[pair] = kStCompleted;
    p.ops_len[pair] = out_n;
    if (p.end_info) {
      p.end_info[3 * (int64_t)pair] = plen;
      p.end_info[3 * (int64_t)pair + 1] = tlen;
      p.end_info[3 * (int64_t)pair + 2] = S;
    }
  }
  return !bad;
}

}  // namespace wf2g

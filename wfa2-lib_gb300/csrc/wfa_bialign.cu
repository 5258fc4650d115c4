// wfa_bialign.cu -- sm_103a kernels of the BiWFA (ultralow memory) path.
//
// Breakpoint search, one CTA per segment (threads striped over diagonals):
//   forward/reverse  two score-only WFAs of the segment, the reverse one on
//                    the reversed sequences and with swapped end components
//                    (wavefront/wavefront_bialign.c:81-150); each keeps the
//                    last max_score_scope wavefronts of every component
//   phase 1          alternate forward/reverse steps until their largest
//                    extended antidiagonals meet (:1000-1041, max antidiagonal
//                    of wavefront/wavefront_extend_kernels.c:125-152)
//   phase 2          overlap checks of the newest wavefront of one side against
//                    the last max_score_scope of the other (:878-956), each
//                    check scanning the shared diagonals for the lowest k
//                    (m2m :798-874, indel2indel :477-573), until the lower
//                    bound passes the best breakpoint (:1043-1082)
// Recursion, base cases and CIGAR assembly run on the host side of the engine
// (wfa_bialign_host.cu); base cases use the unidirectional kernel.
//
// Compute, trims and termination are those of the unidirectional kernel
// (wfa_kernels.cu), on int32 rows, with begin/end components
// (wavefront/wavefront_aligner.c:311-382, wavefront/wavefront_termination.c:37-108).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "wfa_bialign.cuh"

namespace wf2g {

namespace {

constexpr int kBiMaxThreads = 512;
constexpr int kBiMaxWarps = kBiMaxThreads / 32;
constexpr int kRed = 12;  // per step: (trimmed lo, hi) x 5 components, max antidiagonal, edit pruning

struct BiShared {
  int red[2][kBiMaxWarps][kRed];  // per-warp partials, alternating per step
  int res[2][2];  // per step parity: termination flag, max antidiagonal
  int found[3];
  int seg;
};

struct BP {
  int score, score_f, score_r, k_f, off_f, comp;
};

__device__ __forceinline__ uint32_t win2(const uint32_t* W, int pos) {
  const int w = pos >> 4;
  return __funnelshift_l(W[w + 1], W[w], (pos & 15) << 1);
}

template <bool A2P>
struct BiCtx {
  static constexpr int NC = A2P ? 5 : 3;
  const BiParams& p;
  BiShared& sh;
  int2* meta;
  int32_t* rows;
  int tid, nt, lane, warp, nwarps;
  int scope, stride, kofs, kmin, kmax;
  int ext_lo, ext_hi;  // diagonals NULL-initialised in every row of this CTA
  int jfound;
  int rsel;      // which sh.res / sh.red buffer is written next (alternates)
  bool one_bar;  // every input of a step lies >= 2 scores back
  // segment
  int plen, tlen, k_end;
  int enc2;
  const uint32_t* PW;
  const uint32_t* TW;
  const uint8_t* PB;
  const uint8_t* TB;
  int pb, pe, tb, te;
  int s[2], nulls[2], beg[2], endc[2];
  // heuristic state per direction (wavefront_heuristic_t's internals): the
  // wait counter, and x-drop's best score so far and its diagonal
  // (INT_MAX: none yet)
  int steps_wait[2], max_sw[2], max_sw_k[2];
  int2* imeta;        // initialised windows (rows are NULL outside them)

  __device__ BiCtx(const BiParams& p_, BiShared& sh_, int2* meta_)
      : p(p_), sh(sh_), meta(meta_) {
    tid = threadIdx.x;
    nt = blockDim.x;
    lane = tid & 31;
    warp = tid >> 5;
    nwarps = nt >> 5;
    scope = p.scope;
    stride = p.stride;
    kofs = p.kofs;
    kmin = -kofs;
    kmax = stride - kofs - 1;
    rows = p.rows + (int64_t)blockIdx.x * p.rows_per_cta;
    imeta = meta + 2 * NC * p.scope;
    ext_lo = 1;
    ext_hi = 0;
    jfound = 0;
    rsel = 0;
    const Penalties& pen = p.pen;
    int gap = min(pen.x, pen.e1);
    if (A2P) gap = min(gap, pen.e2);
    one_bar = gap >= 2;
  }

  __device__ __forceinline__ int32_t* row(int d, int c, int slot) const {
    return rows + (int64_t)((d * NC + c) * scope + slot) * stride + kofs;
  }
  __device__ __forceinline__ const int32_t* null_row() const {
    return rows + (int64_t)(2 * NC * scope) * stride + kofs;
  }
  // limits (lo,hi) of row (d,c,slot); lo > hi: null
  __device__ __forceinline__ int2& mt(int d, int c, int slot) const {
    return meta[(d * NC + c) * scope + slot];
  }
  // initialised window of the row: equal to the limits except after a
  // heuristic cut-off, which narrows only the limits
  __device__ __forceinline__ int2& wm(int d, int c, int slot) const {
    return imeta[(d * NC + c) * scope + slot];
  }

  // ------------------------------------------------------------ sequences
  // Forward: P[pb+v+i] against T[tb+h+i]; reverse: P[pe-1-v-i] against
  // T[te-1-h-i]; at most lim characters.
  __device__ int lcp(int d, int v, int h, int lim) const {
    int L = 0;
    if (enc2) {
      if (d == 0) {
        const int ps = pb + v + 16, ts = tb + h + 16;
        while (L < lim) {
          const uint32_t x = win2(PW, ps + L) ^ win2(TW, ts + L);
          if (x) {
            L += __clz(x) >> 1;
            break;
          }
          L += 16;
        }
      } else {
        // the 16 bases ending at pattern position pe-1-v-L start at stored
        // position (pe-1-v-L) - 15 + 16
        const int ps = pe - v, ts = te - h;
        while (L < lim) {
          const uint32_t x = win2(PW, ps - L) ^ win2(TW, ts - L);
          if (x) {
            L += (__ffs(x) - 1) >> 1;
            break;
          }
          L += 16;
        }
      }
      return L < lim ? L : lim;
    }
    if (d == 0) {
      const uint8_t* P = PB + pb + v;
      const uint8_t* T = TB + tb + h;
      while (L < lim && P[L] == T[L]) ++L;
    } else {
      const uint8_t* P = PB + (pe - 1 - v);
      const uint8_t* T = TB + (te - 1 - h);
      while (L < lim && P[-L] == T[-L]) ++L;
    }
    return L;
  }

  // First 16-base window of an extension from (v,h), XORed (ACGT pairs).
  __device__ __forceinline__ uint32_t first_window(int d, int v, int h) const {
    if (d == 0) return win2(PW, pb + v + 16) ^ win2(TW, tb + h + 16);
    return win2(PW, pe - v) ^ win2(TW, te - h);
  }
  // Equal characters at the start of a non-zero window XOR.
  __device__ __forceinline__ int eq_count(int d, uint32_t x) const {
    return d == 0 ? (__clz(x) >> 1) : ((__ffs(x) - 1) >> 1);
  }
  // lcp of ACGT pairs from L already-equal characters on.
  __device__ int lcp_from(int d, int v, int h, int L, int lim) const {
    if (d == 0) {
      const int ps = pb + v + 16, ts = tb + h + 16;
      while (L < lim) {
        const uint32_t x = win2(PW, ps + L) ^ win2(TW, ts + L);
        if (x) {
          L += __clz(x) >> 1;
          break;
        }
        L += 16;
      }
    } else {
      const int ps = pe - v, ts = te - h;
      while (L < lim) {
        const uint32_t x = win2(PW, ps - L) ^ win2(TW, ts - L);
        if (x) {
          L += (__ffs(x) - 1) >> 1;
          break;
        }
        L += 16;
      }
    }
    return L < lim ? L : lim;
  }

  // ------------------------------------------------------------ row upkeep
  __device__ void null_range(int32_t* r, int a, int b) const {
    for (int k = a + tid; k <= b; k += nt) r[k] = kNull;
  }
  __device__ void null_range_warp(int32_t* r, int a, int b) const {
    for (int k = a + lane; k <= b; k += 32) r[k] = kNull;
  }
  __device__ void fill_columns(int a, int b) const {
    if (a > b) return;
    const int w = b - a + 1;
    const int64_t nr = 2 * NC * scope + 1;
    const int64_t total = nr * w;
    for (int64_t i = tid; i < total; i += nt) {
      const int64_t r = i / w;
      const int k = a + (int)(i - r * w);
      rows[r * stride + kofs + k] = kNull;
    }
  }
  // Every row is NULL on [a,b] outside its trimmed range after this call.
  // Returns false if [a,b] leaves the rows (never expected).
  __device__ bool ensure_extent(int a, int b) {
    if (a >= ext_lo && b <= ext_hi) return true;
    if (a < kmin || b > kmax) return false;
    if (ext_lo > ext_hi) {
      const int nlo = max(a - 256, kmin), nhi = min(b + 256, kmax);
      fill_columns(nlo, nhi);
      ext_lo = nlo;
      ext_hi = nhi;
    } else {
      const int nlo = a < ext_lo ? max(a - 1024, kmin) : ext_lo;
      const int nhi = b > ext_hi ? min(b + 1024, kmax) : ext_hi;
      fill_columns(nlo, ext_lo - 1);
      fill_columns(ext_hi + 1, nhi);
      ext_lo = nlo;
      ext_hi = nhi;
    }
    __syncthreads();
    return true;
  }

  // ------------------------------------------------------------ one score step
  // Computes wavefront s+1 of direction d, extends it and checks termination.
  // Returns 0 (continue), 1 (end reached), 2 (unreachable), 3 (guard).
  __device__ int step(int d, int& mak_out) {
    const Penalties& pen = p.pen;
    const int s1 = s[d] + 1;
    const int slot = s1 % scope;
    const int2 E = make_int2(1, 0);
    // single-component metrics (wavefront/wavefront_compute_edit.c,
    // wavefront/wavefront_compute_linear.c): no I/D inputs; indel has no
    // mismatch; end-to-end edit prunes wide wavefronts
    const bool lin = p.metric <= 2;
    const bool prune = p.metric == 1;
    auto in = [&](int c, int sc) -> int2 { return sc >= 0 ? mt(d, c, sc % scope) : E; };
    const int2 eMx = p.metric != 0 ? in(kCompM, s1 - pen.x) : E;
    const int2 eMo1 = in(kCompM, s1 - pen.o1 - pen.e1);
    const int2 eI1 = lin ? E : in(kCompI1, s1 - pen.e1);
    const int2 eD1 = lin ? E : in(kCompD1, s1 - pen.e1);
    int2 eMo2 = E, eI2 = E, eD2 = E;
    if (A2P) {
      eMo2 = in(kCompM, s1 - pen.o2 - pen.e2);
      eI2 = in(kCompI2, s1 - pen.e2);
      eD2 = in(kCompD2, s1 - pen.e2);
    }
    const bool vMx = eMx.x <= eMx.y, vMo1 = eMo1.x <= eMo1.y;
    const bool vI1 = eI1.x <= eI1.y, vD1 = eD1.x <= eD1.y;
    const bool vMo2 = A2P && eMo2.x <= eMo2.y;
    const bool vI2 = A2P && eI2.x <= eI2.y, vD2 = A2P && eD2.x <= eD2.y;
    int2 old[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) old[c] = wm(d, c, slot);
    s[d] = s1;

    // wavefront/wavefront_compute_affine.c:236-243: all inputs null
    if (!(vMx | vMo1 | vI1 | vD1 | vMo2 | vI2 | vD2)) {
      ++nulls[d];
#pragma unroll
      for (int c = 0; c < NC; ++c) null_range(row(d, c, slot), old[c].x, old[c].y);
      __syncthreads();
      if (tid == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) mt(d, c, slot) = wm(d, c, slot) = E;
      }
      __syncthreads();
      mak_out = 0;
      // wavefront/wavefront_extend.c:183-192.  Edit and indel with a step
      // limit run on: the reference's edit driver allocates every wavefront,
      // so its null-step count never ends them, only the step limit does.
      return nulls[d] > scope && !edit_runs_on() ? 2 : 0;
    }
    nulls[d] = 0;

    // wavefront/wavefront_compute.c:40-87: output range
    int lo = INT_MAX, hi = INT_MIN;
    if (p.heur && p.metric >= 2) {
      // The reference widens the range by every input, a null one with the
      // all-NULL wavefront's limits [1,-1] (wavefront/wavefront.c:110-117),
      // so the range reaches diagonal 0.  Exact runs read only NULLs out
      // there; under a cut-off the rows' windows can still hold cells.
      const int2 nl = make_int2(1, -1);
      const int2 lMx = vMx ? eMx : nl, lMo1 = vMo1 ? eMo1 : nl;
      lo = min(lMx.x, lMo1.x - 1);
      hi = max(lMx.y, lMo1.y + 1);
      if (!lin) {  // gap-linear stops at the mismatch and open inputs
        const int2 lI1 = vI1 ? eI1 : nl, lD1 = vD1 ? eD1 : nl;
        lo = min(lo, min(lI1.x + 1, lD1.x - 1));
        hi = max(hi, max(lI1.y + 1, lD1.y - 1));
      }
      if (A2P) {
        const int2 lMo2 = vMo2 ? eMo2 : nl, lI2 = vI2 ? eI2 : nl, lD2 = vD2 ? eD2 : nl;
        lo = min(lo, min(lMo2.x - 1, min(lI2.x + 1, lD2.x - 1)));
        hi = max(hi, max(lMo2.y + 1, max(lI2.y + 1, lD2.y - 1)));
      }
    } else {
      if (vMx) { lo = min(lo, eMx.x); hi = max(hi, eMx.y); }
      if (vMo1) { lo = min(lo, eMo1.x - 1); hi = max(hi, eMo1.y + 1); }
      if (vI1) { lo = min(lo, eI1.x + 1); hi = max(hi, eI1.y + 1); }
      if (vD1) { lo = min(lo, eD1.x - 1); hi = max(hi, eD1.y - 1); }
      if (A2P) {
        if (vMo2) { lo = min(lo, eMo2.x - 1); hi = max(hi, eMo2.y + 1); }
        if (vI2) { lo = min(lo, eI2.x + 1); hi = max(hi, eI2.y + 1); }
        if (vD2) { lo = min(lo, eD2.x - 1); hi = max(hi, eD2.y - 1); }
      }
    }
    if (!ensure_extent(lo - 1, hi + 1)) return 3;
    // what the reused slots hold outside [lo,hi]
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (old[c].x <= old[c].y) {
        null_range(row(d, c, slot), old[c].x, min(old[c].y, lo - 1));
        null_range(row(d, c, slot), max(old[c].x, hi + 1), old[c].y);
      }
    }
    const int32_t* const nr = null_row();
    const int32_t* const rMx = vMx ? row(d, kCompM, (s1 - pen.x) % scope) : nr;
    const int32_t* const rMo1 = vMo1 ? row(d, kCompM, (s1 - pen.o1 - pen.e1) % scope) : nr;
    const int32_t* const rI1 = vI1 ? row(d, kCompI1, (s1 - pen.e1) % scope) : nr;
    const int32_t* const rD1 = vD1 ? row(d, kCompD1, (s1 - pen.e1) % scope) : nr;
    const int32_t* rMo2 = nr;
    const int32_t* rI2 = nr;
    const int32_t* rD2 = nr;
    if (A2P) {
      if (vMo2) rMo2 = row(d, kCompM, (s1 - pen.o2 - pen.e2) % scope);
      if (vI2) rI2 = row(d, kCompI2, (s1 - pen.e2) % scope);
      if (vD2) rD2 = row(d, kCompD2, (s1 - pen.e2) % scope);
    }
    // edit and indel NULL the two elements beyond each end of M[s-1]
    // (wavefront/wavefront_compute_edit.c:352-356): only cells a cut-off left
    // in the initialised window can hold values there
    if (p.heur && p.metric <= 1 && vMo1) {
      if (tid == 0) {
        const int sl = (s1 - pen.o1) % scope;
        const int2 w = wm(d, kCompM, sl);
        int32_t* const r = row(d, kCompM, sl);
        const int ks[4] = {eMo1.x - 2, eMo1.x - 1, eMo1.y + 1, eMo1.y + 2};
        for (int j = 0; j < 4; ++j)
          if (ks[j] >= w.x && ks[j] <= w.y) r[ks[j]] = kNull;
      }
      __syncthreads();
    }
    int32_t* const oM = row(d, kCompM, slot);
    int32_t* const oI1 = row(d, kCompI1, slot);
    int32_t* const oD1 = row(d, kCompD1, slot);
    int32_t* const oI2 = A2P ? row(d, kCompI2, slot) : nullptr;
    int32_t* const oD2 = A2P ? row(d, kCompD2, slot) : nullptr;

    int tl[NC], th[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      tl[c] = INT_MAX;
      th[c] = INT_MIN;
    }
    int mak = 0;
    int wmin = INT_MAX;  // edit pruning: best worst case over the unextended cells
    // kU cells per thread per iteration: every input load of the group is
    // issued before the first compute, and the first extend window of each
    // M cell is fetched for the whole group before any is compared
    constexpr int kU = 4;
    for (int kb = lo + tid; kb <= hi; kb += kU * nt) {
      int32_t bestv[kU], i1v[kU], d1v[kU], i2v[kU], d2v[kU];
      bool live[kU];
#pragma unroll
      for (int j = 0; j < kU; ++j) {
        const int k = kb + j * nt;
        live[j] = k <= hi;
        const int kk = live[j] ? k : lo;  // in-range stand-in for cells past hi
        // wavefront/wavefront_compute_affine.c:66-84
        const int32_t i1 = max(rMo1[kk - 1], rI1[kk - 1]) + 1;
        const int32_t d1 = max(rMo1[kk + 1], rD1[kk + 1]);
        const int32_t mis = rMx[kk] + 1;
        int32_t ins = i1, del = d1;
        int32_t i2 = kNull, d2 = kNull;
        if (A2P) {
          // wavefront/wavefront_compute_affine2p.c:78-95
          i2 = max(rMo2[kk - 1], rI2[kk - 1]) + 1;
          d2 = max(rMo2[kk + 1], rD2[kk + 1]);
          ins = max(i1, i2);
          del = max(d1, d2);
        }
        bestv[j] = max(del, max(mis, ins));
        i1v[j] = i1;
        d1v[j] = d1;
        i2v[j] = i2;
        d2v[j] = d2;
      }
      uint32_t xw[kU];
      bool okm[kU];
#pragma unroll
      for (int j = 0; j < kU; ++j) {
        const int k = kb + j * nt;
        const int32_t best = bestv[j];
        // M out of bounds -> NULL
        okm[j] = live[j] && (uint32_t)best <= (uint32_t)tlen &&
                 (uint32_t)(best - k) <= (uint32_t)plen;
        xw[j] = enc2 ? first_window(d, okm[j] ? best - k : 0, okm[j] ? best : 0) : 0u;
      }
#pragma unroll
      for (int j = 0; j < kU; ++j) {
        if (!live[j]) continue;
        const int k = kb + j * nt;
        const int32_t best = bestv[j], i1 = i1v[j], d1 = d1v[j];
        // trims of wavefront/wavefront_compute.c:579-613
        const bool okI1 = (uint32_t)i1 <= (uint32_t)tlen;
        const bool okD1 = (uint32_t)(d1 - k) <= (uint32_t)plen;
        int32_t mext = kNull;
        if (okm[j]) {
          const int v = best - k;
          if (prune) wmin = min(wmin, max(plen - v, tlen - best));
          const int lim = min(plen - v, tlen - best);
          int L;
          if (!enc2) L = lcp(d, v, best, lim);
          else if (xw[j]) L = min(eq_count(d, xw[j]), lim);
          else L = lim <= 16 ? lim : lcp_from(d, v, best, 16, lim);
          mext = best + L;
          mak = max(mak, 2 * mext - k);
        }
        oM[k] = mext;
        oI1[k] = i1;
        oD1[k] = d1;
        if (okm[j]) { tl[0] = min(tl[0], k); th[0] = k; }
        if (okI1) { tl[1] = min(tl[1], k); th[1] = k; }
        if (okD1) { tl[2] = min(tl[2], k); th[2] = k; }
        if (A2P) {
          const int32_t i2 = i2v[j], d2 = d2v[j];
          oI2[k] = i2;
          oD2[k] = d2;
          if ((uint32_t)i2 <= (uint32_t)tlen) { tl[NC - 2] = min(tl[NC - 2], k); th[NC - 2] = k; }
          if ((uint32_t)(d2 - k) <= (uint32_t)plen) { tl[NC - 1] = min(tl[NC - 1], k); th[NC - 1] = k; }
        }
      }
    }
    // block reductions: per-warp partials, then warp 0
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      tl[c] = __reduce_min_sync(kFull, tl[c]);
      th[c] = __reduce_max_sync(kFull, th[c]);
    }
    mak = __reduce_max_sync(kFull, mak);
    if (prune) wmin = __reduce_min_sync(kFull, wmin);
    // partials of this step in buffer rsel: a warp reads them after the
    // barrier below and writes the other buffer next step, and no warp can
    // write this buffer again before every warp passed the next barrier
    int (*red)[kRed] = sh.red[rsel];
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        red[warp][2 * c] = tl[c];
        red[warp][2 * c + 1] = th[c];
      }
      red[warp][2 * NC] = mak;
      red[warp][2 * NC + 1] = wmin;
    }
    __syncthreads();
    // every warp reduces the partials itself (the same values everywhere)
    int v = 0;
    if (lane <= 2 * NC + 1) {
      const bool is_lo = (lane < 2 * NC && !(lane & 1)) || lane == 2 * NC + 1;
      v = red[0][lane];
      for (int w = 1; w < nwarps; ++w) {
        const int x = red[w][lane];
        v = is_lo ? min(v, x) : max(v, x);
      }
    }
    rsel ^= 1;
    int2 nm[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const int a = __shfl_sync(kFull, v, 2 * c);
      const int b = __shfl_sync(kFull, v, 2 * c + 1);
      nm[c] = a > b ? E : make_int2(a, b);
    }
    const int mk = __shfl_sync(kFull, v, 2 * NC);
    if (lin) nm[kCompI1] = nm[kCompD1] = E;  // one component: no gap wavefronts
    if (prune && nm[kCompM].y - nm[kCompM].x + 1 >= 1000) {
      // exact pruning of a wide edit wavefront on its unextended offsets
      // (wavefront/wavefront_compute_edit.c:220-279); every thread derives
      // the same limits
      const int wm_ = __shfl_sync(kFull, v, 2 * NC + 1);
      const int tlo = nm[kCompM].x, thi = nm[kCompM].y;
      const int sk = tlo + (thi - tlo) / 2;
      int32_t so = max(rMo1[sk + 1], max(rMx[sk], rMo1[sk - 1]) + 1);
      if (!((uint32_t)so <= (uint32_t)tlen && (uint32_t)(so - sk) <= (uint32_t)plen)) so = -1;
      if (so >= 0) {
        const int smax = max(plen - (so - sk), tlen - so);
        if (!(abs(tlo - k_end) <= smax && abs(thi - k_end) <= smax)) {
          const int a = max(tlo, k_end - wm_);
          const int nlo = (a <= min(thi, k_end + wm_)) ? a : thi + 1;
          const int b = min(thi, k_end + wm_);
          const int nhi = (b > nlo && b >= k_end - wm_) ? b : nlo;
          nm[kCompM] = nlo > nhi ? E : make_int2(nlo, nhi);
        }
      }
    }
    // warp 0 NULLs the trimmed ends and publishes the limits; the next step
    // reads neither when every input lies two or more scores back (one_bar),
    // otherwise a second barrier orders them
    if (warp == 0) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        int32_t* const r = row(d, c, slot);
        if (nm[c].x > nm[c].y) {
          null_range_warp(r, lo, hi);
        } else {
          null_range_warp(r, lo, nm[c].x - 1);
          null_range_warp(r, nm[c].y + 1, hi);
        }
      }
      if (lane == 0) {
#pragma unroll
        for (int c = 0; c < NC; ++c) mt(d, c, slot) = wm(d, c, slot) = nm[c];
      }
    }
    // wavefront/wavefront_termination.c:37-108 on the end component
    const int ec = endc[d];
    const int2 em = nm[ec];
    const int flag =
        (em.x <= k_end && k_end <= em.y && row(d, ec, slot)[k_end] >= tlen) ? 1 : 0;
    if (p.heur && !flag) cutoff(d, slot, nm[kCompM]);
    if (!one_bar) __syncthreads();
    mak_out = flag ? 0 : mk;
    return flag;
  }

  // Score-0 extension (wavefront/wavefront_extend.c:173-211): only where the
  // direction begins in M.
  __device__ int extend0(int d, int& mak_out) {
    mak_out = 0;
    if (beg[d] != kCompM) return 0;
    if (tid == 0) {
      const int L = lcp(d, 0, 0, min(plen, tlen));
      row(d, kCompM, 0)[0] = L;
      sh.res[rsel][0] = (endc[d] == kCompM && k_end == 0 && L >= tlen) ? 1 : 0;
      sh.res[rsel][1] = 2 * L;
    }
    __syncthreads();
    const int flag = sh.res[rsel][0];
    mak_out = flag ? 0 : sh.res[rsel][1];
    rsel ^= 1;
    if (p.heur && !flag) cutoff(d, 0, make_int2(0, 0));
    return flag;
  }

  // Heuristic cut-off of M at `slot` after its extension
  // (wavefront/wavefront_heuristic.c:506-563): one of wf-adaptive / wfmash,
  // x-drop, one of banded static / adaptive, sharing one wait counter (z-drop
  // is not computed here); block-uniform.  Only limits shrink (M, and the I/D
  // rows of the score intersected with M); the cut cells stay in the rows'
  // initialised windows.
  __device__ void cutoff(int d, int slot, int2 mlim) {
    if (mlim.x > mlim.y) return;  // empty M: no step counted
    --steps_wait[d];
    const int hs = p.heur;
    const int mlo = mlim.x, mhi = mlim.y;
    int nlo = mlo, nhi = mhi;
    const int32_t* const mr = row(d, kCompM, slot);
    // wf-adaptive / wfmash (:229-289): cells further from the end than the
    // closest by more than max_distance_threshold, from both ends, keeping the
    // end diagonal's side
    if ((hs & (kHsWfadaptive | kHsWfmash)) && steps_wait[d] <= 0 && nhi - nlo + 1 >= p.h_min_len) {
      const bool wmash = !(hs & kHsWfadaptive);
      // wfmash weighs each side by its length (:134-145), in float as the
      // reference does
      const int mfactor = wmash ? __float2int_rz(__fdiv_rn((float)(plen + tlen), 2.0f)) : 0;
      auto dist = [&](int k) -> int {
        const int32_t off = mr[k];
        if (off < 0) return 1 << 30;
        if (!wmash) return max(plen - (off - k), tlen - off);
        const int lv = __float2int_rz(
            __fmul_rn(__fdiv_rn((float)(plen - (off - k)), (float)plen), (float)mfactor));
        const int lh = __float2int_rz(
            __fmul_rn(__fdiv_rn((float)(tlen - off), (float)tlen), (float)mfactor));
        return max(lv, lh);
      };
      int dm = max(plen, tlen);
      for (int k = nlo + tid; k <= nhi; k += nt) dm = min(dm, dist(k));
      dm = block_min(dm);
      const int top = min(k_end, nhi);
      int first = INT_MAX;
      for (int k = nlo + tid; k < top; k += nt)
        if (dist(k) - dm <= p.h_max_dist) { first = k; break; }
      first = block_min(first);
      const int wlo = first == INT_MAX ? max(nlo, top) : first;
      const int bot = max(k_end, wlo);
      int neg_last = INT_MAX;  // -(last qualifying k), for a block minimum
      for (int k = nhi - tid; k > bot; k -= nt)
        if (dist(k) - dm <= p.h_max_dist) { neg_last = -k; break; }
      neg_last = block_min(neg_last);
      nhi = neg_last == INT_MAX ? min(nhi, bot) : -neg_last;
      nlo = wlo;
      steps_wait[d] = p.h_steps;
    }
    // x-drop (:326-380) on the cells' SW scores (wavefront/wavefront_penalties.h:73)
    // at this direction's score, with the first best cell
    if ((hs & kHsXdrop) && steps_wait[d] <= 0) {
      const int swg = p.pen.match != 0 ? -p.pen.match : -1;
      const int sd = s[d];
      auto sw = [&](int k, int32_t off) -> int { return (swg * (2 * off - k) - sd) / 2; };
      int tbest = INT_MIN, tk = INT_MAX;
      for (int k = nlo + tid; k <= nhi; k += nt) {
        const int32_t off = mr[k];
        if (off < 0) continue;
        const int sc = sw(k, off);
        if (sc > tbest) { tbest = sc; tk = k; }
      }
      const int cmax = block_max(tbest);
      int cmax_k = block_min(tbest == cmax ? tk : INT_MAX);
      if (cmax == INT_MIN) cmax_k = 0;
      if (max_sw_k[d] != INT_MAX) {
        // cells xdrop or more below the best seen are cut from both ends
        const int best = max_sw[d];
        auto keep = [&](int k) -> bool {
          const int32_t off = mr[k];
          return off >= 0 && (int)((uint32_t)best - (uint32_t)sw(k, off)) < p.h_xdrop;
        };
        int first = INT_MAX;
        for (int k = nlo + tid; k <= nhi; k += nt)
          if (keep(k)) { first = k; break; }
        first = block_min(first);
        const int xlo = first == INT_MAX ? nhi + 1 : first;
        int neg_last = INT_MAX;
        for (int k = nhi - tid; k >= xlo; k -= nt)
          if (keep(k)) { neg_last = -k; break; }
        neg_last = block_min(neg_last);
        if (xlo <= nhi) nhi = -neg_last;
        nlo = xlo;
        if (cmax > max_sw[d]) {
          max_sw[d] = cmax;
          max_sw_k[d] = cmax_k;
        }
      } else {
        max_sw[d] = cmax;
        max_sw_k[d] = cmax_k;
      }
      steps_wait[d] = p.h_steps;
    }
    // banded (:451-505)
    if (hs & kHsBandedStatic) {
      nlo = max(nlo, p.h_min_k);
      nhi = min(nhi, p.h_max_k);
    } else if ((hs & kHsBandedAdaptive) && steps_wait[d] <= 0 && nhi - nlo + 1 >= 4) {
      const int len = nhi - nlo + 1, maxlen = p.h_max_k - p.h_min_k + 1;
      if (len > maxlen) {
        // place the band by the distances of four sampled cells
        auto dist = [&](int k) -> int {
          const int32_t off = mr[k];
          return off >= 0 ? max(plen - (off - k), tlen - off) : (1 << 30);
        };
        const int leeway = (len - maxlen) / 2, quarter = len / 4;
        int blo = nlo;
        if (dist(nlo) > dist(nhi)) blo += leeway;
        if (dist(nlo + quarter) > dist(nlo + 2 * quarter)) blo += leeway;
        nhi = min(blo + maxlen - 1, nhi);
        nlo = max(blo, nlo);
      }
      steps_wait[d] = p.h_steps;
    }
    if (nlo == mlo && nhi == mhi) return;
    if (tid == 0) {
      mt(d, kCompM, slot) = make_int2(nlo, nhi);
      for (int c = 1; c < NC; ++c) {
        const int2 m = mt(d, c, slot);
        mt(d, c, slot) = make_int2(max(m.x, nlo), min(m.y, nhi));
      }
    }
  }

  // ------------------------------------------------------------ overlap
  __device__ int block_max(int v) { return ~block_min(~v); }

  __device__ int block_min(int v) {
    v = __reduce_min_sync(kFull, v);
    const int j = jfound % 3;
    if (lane == 0 && v != INT_MAX) atomicMin(&sh.found[j], v);
    __syncthreads();
    const int r = sh.found[j];
    if (tid == 0) sh.found[(j + 2) % 3] = INT_MAX;
    ++jfound;
    return r;
  }

  // One breakpoint check of component c between wavefront score_0 of side d0
  // and wavefront score_1 of the other side.
  __device__ void check(int d0, int c, int score_0, int score_1, bool forward, bool indel,
                        int gap_open, BP& bp) {
    const int d1 = d0 ^ 1;
    const int2 m0 = mt(d0, c, score_0 % scope);
    const int2 m1 = mt(d1, c, score_1 % scope);
    if (m0.x > m0.y || m1.x > m1.y) return;
    const int lo_0 = m0.x, hi_0 = m0.y;
    const int lo_1 = tlen - plen - m1.y, hi_1 = tlen - plen - m1.x;
    if (hi_1 < lo_0 || hi_0 < lo_1) return;
    if (score_0 + score_1 - (indel ? gap_open : 0) >= bp.score) return;
    const int min_hi = min(hi_0, hi_1), max_lo = max(lo_0, lo_1);
    const int32_t* const r0 = row(d0, c, score_0 % scope);
    const int32_t* const r1 = row(d1, c, score_1 % scope);
    int found = INT_MAX;
    for (int k0 = max_lo + tid; k0 <= min_hi; k0 += nt) {
      const int k1 = tlen - plen - k0;
      const int32_t o0 = r0[k0], o1 = r1[k1];
      if (o0 + o1 >= tlen) {
        if (indel) {
          // only the forward side is bounds-checked (wavefront/wavefront_bialign.c:549-561)
          if (forward) {
            if (o0 - k0 > plen || o0 > tlen) continue;
          } else {
            if (o1 - k1 > plen || o1 > tlen) continue;
          }
        }
        found = k0;
        break;
      }
    }
    found = block_min(found);
    if (found == INT_MAX) return;
    const int k0 = found, k1 = tlen - plen - k0;
    const int32_t o0 = r0[k0], o1 = r1[k1];
    if (forward) {
      bp.score_f = score_0;
      bp.score_r = score_1;
      bp.k_f = k0;
      bp.off_f = o0;
    } else {
      bp.score_f = score_1;
      bp.score_r = score_0;
      bp.k_f = k1;
      bp.off_f = o1;
    }
    bp.score = score_0 + score_1 - (indel ? gap_open : 0);
    bp.comp = c;
  }

  // wavefront/wavefront_bialign.c:878-956
  __device__ void overlap(int d0, bool forward, BP& bp) {
    __syncthreads();  // the last step's trimmed ends and limits are in place
    const Penalties& pen = p.pen;
    const int score_0 = s[d0], score_1 = s[d0 ^ 1];
    if (score_0 == 0 && beg[d0] != kCompM) return;  // no M wavefront at score 0
    for (int i = 0; i < scope; ++i) {
      const int si = score_1 - i;
      if (si < 0) break;
      if (A2P) {
        if (score_0 + si - pen.o2 >= bp.score) continue;
        check(d0, kCompD2, score_0, si, forward, true, pen.o2, bp);
        check(d0, kCompI2, score_0, si, forward, true, pen.o2, bp);
      }
      if (score_0 + si - pen.o1 >= bp.score) continue;
      check(d0, kCompD1, score_0, si, forward, true, pen.o1, bp);
      check(d0, kCompI1, score_0, si, forward, true, pen.o1, bp);
      if (score_0 + si >= bp.score) continue;
      check(d0, kCompM, score_0, si, forward, false, 0, bp);
    }
  }

  // ------------------------------------------------------------ one segment
  __device__ void run_segment(int seg) {
    const BiSeg sg = p.segs[seg];
    const int pair = sg.pair;
    enc2 = p.enc2[pair];
    PW = p.packed + p.pk_p[pair];
    TW = p.packed + p.pk_t[pair];
    PB = p.seqs + p.p_off[pair];
    TB = p.seqs + p.t_off[pair];
    pb = sg.pb;
    pe = sg.pe;
    tb = sg.tb;
    te = sg.te;
    plen = pe - pb;
    tlen = te - tb;
    k_end = tlen - plen;
    beg[0] = sg.cb;
    endc[0] = sg.ce;
    beg[1] = sg.ce;
    endc[1] = sg.cb;
    s[0] = s[1] = 0;
    nulls[0] = nulls[1] = 0;
    // wavefront_heuristic_clear at each init (wavefront/wavefront_heuristic.c:114-121)
    steps_wait[0] = steps_wait[1] = p.h_steps;
    max_sw[0] = max_sw[1] = 0;
    max_sw_k[0] = max_sw_k[1] = INT_MAX;
    BiOut res;
    res.status = kBiGuard;
    res.reached = 0;
    res.score = res.score_f = res.score_r = res.k_f = res.off_f = res.comp = 0;
    const int64_t guard64 = (int64_t)scope * ((int64_t)plen + tlen + 2) + 64;
    const int guard = (int)min(guard64, (int64_t)INT_MAX / 2);

    if (ensure_extent(-2, 2)) {
      if (tid == 0) {
        row(0, beg[0], 0)[0] = 0;
        mt(0, beg[0], 0) = wm(0, beg[0], 0) = make_int2(0, 0);
        row(1, beg[1], 0)[0] = 0;
        mt(1, beg[1], 0) = wm(1, beg[1], 0) = make_int2(0, 0);
      }
      __syncthreads();
      search(res, guard);
    }
    if (tid == 0) p.out[seg] = res;
    __syncthreads();  // the last step's trimmed ends and limits are in place
    // leave every row NULL for the next segment
    for (int d = 0; d < 2; ++d)
      for (int c = 0; c < NC; ++c)
        for (int sl = 0; sl < scope; ++sl) {
          const int2 m = wm(d, c, sl);
          if (m.x <= m.y) null_range(row(d, c, sl), m.x, m.y);
        }
    __syncthreads();
    for (int i = tid; i < 4 * NC * scope; i += nt) meta[i] = make_int2(1, 0);
    __syncthreads();
  }

  // Edit and indel with a step limit do not end on null wavefronts.
  __device__ bool edit_runs_on() const { return p.metric <= 1 && p.max_steps != INT_MAX; }

  // Scores past the segment's bound: no alignment scores that high, so an
  // edit or indel search that runs on would reach its step limit.
  __device__ void guard_reached(BiOut& res) {
    if (edit_runs_on()) res.status = kBiMaxSteps;
    else finish(res, 3, 0);
  }

  __device__ void finish(BiOut& res, int r, int d) {
    if (r == 1) {
      res.status = kBiEndReached;
      res.reached = s[d];
    } else if (r == 2) {
      res.status = kBiUnreachable;
    } else {
      res.status = kBiGuard;
    }
  }

  // wavefront/wavefront_bialign.c:975-1083
  __device__ void search(BiOut& res, int guard) {
    int fmax = 0, rmax = 0, mak = 0, r;
    if ((r = extend0(0, fmax))) return finish(res, r, 0);
    if ((r = extend0(1, rmax))) return finish(res, r, 1);
    const int max_ad = plen + tlen - 1;
    bool last_fwd = false;
    while (true) {
      if (fmax + rmax >= max_ad) break;
      r = step(0, mak);
      fmax = max(fmax, mak);
      last_fwd = true;
      if (r) return finish(res, r, 0);
      if (fmax + rmax >= max_ad) break;
      r = step(1, mak);
      rmax = max(rmax, mak);
      last_fwd = false;
      if (r) return finish(res, r, 1);
      if (s[1] + s[0] >= p.max_steps) {
        res.status = kBiMaxSteps;
        return;
      }
      if (s[0] + s[1] > guard) return guard_reached(res);
    }
    // wavefront/wavefront_bialign.c:960-973
    const Penalties& pen = p.pen;
    // wavefront/wavefront_bialign.c:960-973 (0 for the single-component metrics)
    const int gap_opening = A2P ? max(pen.o1, pen.o2) : p.metric == 3 ? pen.o1 : 0;
    BP bp;
    bp.score = INT_MAX;
    bp.score_f = bp.score_r = bp.k_f = bp.off_f = bp.comp = 0;
    while (true) {
      if (last_fwd) {
        const int min_sr = s[1] > scope - 1 ? s[1] - (scope - 1) : 0;
        if (s[0] + min_sr - gap_opening >= bp.score) break;
        overlap(0, true, bp);
        r = step(1, mak);
        if (r) return finish(res, r, 1);
      }
      const int min_sf = s[0] > scope - 1 ? s[0] - (scope - 1) : 0;
      if (min_sf + s[1] - gap_opening >= bp.score) break;
      overlap(1, false, bp);
      r = step(0, mak);
      if (r) return finish(res, r, 0);
      if (s[1] + s[0] >= p.max_steps) {
        res.status = kBiMaxSteps;
        return;
      }
      if (s[0] + s[1] > guard) return guard_reached(res);
      last_fwd = true;
    }
    res.status = kBiOk;
    res.score = bp.score;
    res.score_f = bp.score_f;
    res.score_r = bp.score_r;
    res.k_f = bp.k_f;
    res.off_f = bp.off_f;
    res.comp = bp.comp;
  }
};

}  // namespace

// gap-affine fits 64 registers (two 512-thread CTAs per SM); affine2p keeps 128
template <bool A2P>
__global__ void __launch_bounds__(kBiMaxThreads, A2P ? 1 : 2)
    wfa_bi_breakpoint_kernel(const __grid_constant__ BiParams p) {
  extern __shared__ __align__(16) uint8_t smem[];
  BiShared& sh = *reinterpret_cast<BiShared*>(smem);
  int2* meta = reinterpret_cast<int2*>(smem + ((sizeof(BiShared) + 15) & ~size_t(15)));
  BiCtx<A2P> c(p, sh, meta);
  for (int i = c.tid; i < 4 * BiCtx<A2P>::NC * c.scope; i += c.nt) meta[i] = make_int2(1, 0);
  if (c.tid < 3) sh.found[c.tid] = INT_MAX;
  __syncthreads();
  while (true) {
    if (c.tid == 0) sh.seg = atomicAdd(p.queue, 1);
    __syncthreads();
    const int seg = sh.seg;
    __syncthreads();
    if (seg >= p.nseg) break;
    c.run_segment(seg);
  }
}

template __global__ void wfa_bi_breakpoint_kernel<false>(const __grid_constant__ BiParams p);
template __global__ void wfa_bi_breakpoint_kernel<true>(const __grid_constant__ BiParams p);

// 2-bit packing of every pair (one CTA per pair); enc2[pair] = 0 when a
// sequence holds a byte outside {A,C,G,T} (those pairs compare bytes).
__global__ void wfa_bi_pack_kernel(const PackParams q) {
  for (int pair = blockIdx.x; pair < q.n; pair += gridDim.x) {
    int ok = 1;
    for (int which = 0; which < 2; ++which) {
      const uint8_t* src = q.seqs + (which ? q.t_off[pair] : q.p_off[pair]);
      const int len = which ? q.t_len[pair] : q.p_len[pair];
      uint32_t* W = q.packed + (which ? q.pk_t[pair] : q.pk_p[pair]);
      const int64_t nw = packed_words(len);
      for (int64_t w = threadIdx.x; w < nw; w += blockDim.x) {
        // word w holds bases [16w-16, 16w), first base in the top bits
        const int64_t base0 = 16 * w - 16;
        uint32_t x = 0;
        for (int j = 0; j < 16; ++j) {
          const int64_t i = base0 + j;
          if (i >= 0 && i < len) {
            const uint8_t ch = src[i];
            ok &= (ch == 'A') | (ch == 'C') | (ch == 'G') | (ch == 'T');
            x |= ((uint32_t)(ch >> 1) & 3u) << (30 - 2 * j);  // A0 C1 T2 G3
          }
        }
        W[w] = x;
      }
    }
    ok = __syncthreads_and(ok);
    if (threadIdx.x == 0) q.enc2[pair] = ok ? 1 : 0;
    __syncthreads();
  }
}

// CIGAR assembly: one warp per piece.
__global__ void wfa_bi_gather_kernel(const CopyDesc* __restrict__ d, int n,
                                     const uint8_t* __restrict__ src, uint8_t* __restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = w0; i < n; i += nw) {
    const CopyDesc c = d[i];
    if (c.fill) {
      for (int j = lane; j < c.len; j += 32) dst[c.dst + j] = (uint8_t)c.fill;
    } else {
      for (int j = lane; j < c.len; j += 32) dst[c.dst + j] = src[c.src + j];
    }
  }
}

extern "C" void* wf2g_bi_kernel_ptr(int a2p) {
  return a2p ? (void*)wfa_bi_breakpoint_kernel<true> : (void*)wfa_bi_breakpoint_kernel<false>;
}
extern "C" void* wf2g_bi_pack_ptr(void) { return (void*)wfa_bi_pack_kernel; }
extern "C" void* wf2g_bi_gather_ptr(void) { return (void*)wfa_bi_gather_kernel; }
extern "C" size_t wf2g_bi_smem_bytes(int a2p, int scope) {
  const int nc = a2p ? 5 : 3;
  // limits and initialised windows of every row
  return ((sizeof(BiShared) + 15) & ~size_t(15)) + (size_t)4 * nc * scope * sizeof(int2);
}

}  // namespace wf2g

// wfa_fast.cu -- the shared-memory kernel of the GB300 wavefront aligner for
// the library's headline form: gap-affine, exact (no heuristic), end-to-end,
// A/C/G/T sequences.  It runs first over a batch; a pair it cannot finish
// (non-ACGT bytes, a wavefront wider than its shared-memory rows, a score
// beyond its back-trace rows, a step limit, an unreachable end) goes to a
// retry list that the general kernel (wfa_align.cuh) takes in full, so every
// pair's result is the general kernel's result or this kernel's identical one.
//
// Semantics are the reference's exact unidirectional WFA
// (wavefront/wavefront_unialign.c:242-273):
//   compute  wavefront/wavefront_compute_affine.c:44-86 (unsigned bounds test
//            on M only), limits wavefront/wavefront_compute.c:40-87, trimming
//            of the row ends wavefront/wavefront_compute.c:579-613;
//   extend   wavefront/wavefront_extend.c:86-121 (exact LCP per diagonal);
//   end      wavefront/wavefront_termination.c:37-60 (M[s][tlen-plen] >= tlen);
//   score    wavefront/wavefront_compute.c:108-120 (classic score);
//   CIGAR    wavefront/wavefront_backtrace.c:320-529, reproduced from one
//            4-bit choice code per cell: M takes mismatch > deletion >
//            insertion on ties, a gap takes extension over opening (:49-59).
//
// GPU design (differs from the general kernel where it pays):
//   * Scores are divided by g = gcd(x, o+e, e).  Every wavefront at a score
//     that is not a multiple of g is null in the reference (its inputs lie at
//     scores that are not multiples of g either, down to score 0), so the
//     scaled recurrence visits exactly the non-null wavefronts; with the
//     default (4,6,2) it halves the steps.
//   * One group of G threads per pair (a warp; or two to four warps for the
//     wide pairs of the second pass), threads striped over diagonals.  The
//     wavefront ring lives in shared memory as int16 offsets over W
//     diagonals [-W/2, W/2), so every input of a step is one LDS away and no
//     step waits on L2.  Rows are NULL outside their trimmed limits; the cell
//     loop reads k-1, k, k+1 without checks.  A warp per pair updates its
//     rows in place (max(x,o+e)/g M rows, e/g I and D rows), which keeps its
//     shared memory small enough for about 15 pairs per SM.
//   * Sequences are staged 2 bits per base as 64-bit word pairs (word i and
//     i+1 at every i): a 16-base window is one LDS.64 and one funnel shift.
//   * Choice codes (4 bits per cell, eight cells of a thread per 32-bit word)
//     go to a per-group global slice, one fixed-size row per scaled score,
//     with each row's limits beside them for the back-trace.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <type_traits>

#include "wfa_fast_common.cuh"
#include "wfa_kernels.cuh"

namespace wf2g {

// Per-step parameters the group's first warp publishes to the others.
struct FastStep {
  int flag;                // kStepCells, kStepNull, kStepDone, kStepLeave
  int s;                   // scaled score being computed
  int lo, hi;              // its cells
  int rMx, rMo, rI, rD;    // input rows (element offsets of diagonal 0)
  int oM, oI, oD;          // output rows
  int used_lo, used_hi;    // diagonals the pair has touched (for the next pair's reset)
  int2 oldM, oldI, oldD;   // what the output slots held (cleared after the cells, in place)
};
enum { kStepCells = 0, kStepNull = 1, kStepDone = 2, kStepLeave = 3 };
static_assert(2 * sizeof(FastStep) <= 256, "the engine reserves 256 bytes for the step parameters");

// The fast kernel.  CIGAR: full alignment (choice codes, back-trace, replay)
// or score only.  G: threads per pair (32, 64 or 128), one pair per CTA.  W:
// diagonals per shared-memory row.  The first warp keeps the ring's state and
// does each step's bookkeeping (input limits, range, clears, trimming, the
// end test); every warp computes cells.  With G > 32 the warps meet at two
// CTA barriers per step: after the bookkeeping, and after the cells.
template <bool CIGAR, int G, int W>
__global__ void __launch_bounds__(G) wfa_fast_kernel(const FastParams p) {
  static_assert(G == 32 || G == 64 || G == 128, "one to four warps per pair");
  static_assert(W / G <= 64, "per-thread cell masks hold at most 64 cells per step");
  // One warp per pair updates the rows in place: the M ring holds
  // max(x, o+e) rows and I and D e rows each (the engine sizes it so); a
  // step's output rows are the slots of its oldest inputs.
  constexpr bool INPLACE = (G == 32);
  constexpr int NW = G / 32;
  constexpr int HALF = W / 2;
  constexpr int J = (W + G - 1) / G;     // most iterations of a step
  constexpr int RW = ((J + 7) / 8) * G;  // 32-bit choice words per step (8 cells each)
  // per-thread cell masks: bit j for the thread's cell of iteration j
  typedef typename std::conditional<(J > 32), unsigned long long, uint32_t>::type Mask;
  extern __shared__ __align__(16) uint8_t smem[];
  const int t = threadIdx.x;
  const int lane = t & 31;
  const int wig = t >> 5;
  const int nrows = p.R + 2 * p.RI;
  int16_t* const rows = reinterpret_cast<int16_t*>(smem + p.rows_off);
  uint2* const QP = reinterpret_cast<uint2*>(smem + p.q_off);
  uint2* const QT = QP + p.nq;
  int2* const meta = reinterpret_cast<int2*>(smem + p.meta_off);  // first warp's ring limits
  // the step parameters, double-buffered: after a null step no barrier
  // separates the other warps' reads of one step's parameters from the first
  // warp's writes of the next step's
  FastStep* const info = reinterpret_cast<FastStep*>(smem + p.red_off);
  int32_t* const part = reinterpret_cast<int32_t*>(info + 2);  // [NW][8] partial reductions
  int32_t* const bcast = part + NW * 8;
  // per-group slice: [choice words: s_cap rows of RW][row limits: s_cap short2][walk items]
  uint8_t* const slice = p.scratch + (int64_t)blockIdx.x * p.slice_bytes;
  uint32_t* const codes = reinterpret_cast<uint32_t*>(slice);
  short2* const tab = reinterpret_cast<short2*>(slice + (int64_t)p.s_cap * RW * 4);
  uint8_t* const items = slice + p.items_off;
  const int rowI = p.R, rowD = p.R + p.RI;

  // all rows NULL (two int16 NULLs per 32-bit word)
  {
    uint32_t* const r32 = reinterpret_cast<uint32_t*>(rows);
    for (int i = t; i < nrows * W / 2; i += G) r32[i] = 0x80008000u;
  }
  int used_lo = 0, used_hi = -1;  // diagonals the previous pair touched
  const int n_items = p.num_items_dev ? *p.num_items_dev : p.n_items;

  while (true) {
    // ---------------------------------------------------------- next pair
    int item = 0;
    if (G == 32) {
      if (t == 0) item = atomicAdd(p.queue, 1);
      item = __shfl_sync(kFull, item, 0);
    } else {
      if (t == 0) bcast[0] = atomicAdd(p.queue, 1);
      __syncthreads();
      item = bcast[0];
    }
    if (item >= n_items) break;
    const int pair = p.items ? p.items[item] : item;
    const int plen = p.p_len[pair];
    const int tlen = p.t_len[pair];
    auto punt = [&]() {
      if (t == 0) p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
    };

    // ---------------------------------------------------------- reset
    if (used_lo <= used_hi) {
      // word-aligned span of the touched diagonals, in every row
      const int a = (used_lo + HALF) >> 1, b = (used_hi + HALF) >> 1;
      const int span = b - a + 1;
      uint32_t* const r32 = reinterpret_cast<uint32_t*>(rows);
      for (int i = t; i < nrows * span; i += G) {
        const int r = i / span, j = i - r * span;
        r32[r * (W / 2) + a + j] = 0x80008000u;
      }
    }
    if (wig == 0)
      for (int r = lane; r < nrows; r += 32) meta[r] = make_int2(1, 0);
    // (a sequence over the bound is not staged past nq words: it is punted below)
    bool ok = fast_stage<G>(p.seqs + p.p_off[pair], min(plen, p.max_len), QP, p.nq, t);
    ok &= fast_stage<G>(p.seqs + p.t_off[pair], min(tlen, p.max_len), QT, p.nq, t);
    fast_sync<G>();
    const int k_end = tlen - plen;
    // longer than the batch's stated bound (the staged words would not hold
    // it) or ending on a diagonal the rows do not hold: the general kernel
    if (!ok || plen > p.max_len || tlen > p.max_len || k_end < 1 - HALF || k_end > HALF - 2) {
      punt();
      used_lo = 0;
      used_hi = -1;
      fast_sync<G>();
      continue;
    }

    // ---------------------------------------------------------- score 0
    // M[0][0] = 0, extended at once (wavefront/wavefront_aligner.c:311-382)
    const int L0 = fast_lcp(QP, QT, 0, 0, min(plen, tlen));
    // state of the first warp (every lane alike)
    int s = 0;           // scaled score of the last computed wavefront
    int cM = 0, cI = 0;  // its ring slots
    int null_steps = 0;
    int64_t bt_used = 0;     // choice codes of the pair: the general kernel's byte count
    int w_lo = 0, w_hi = 0;  // diagonals touched
    bool done = (plen == tlen) && (L0 >= tlen);
    if (wig == 0 && lane == 0) {
      rows[HALF] = (int16_t)L0;  // row 0 (slot 0 of M), diagonal 0
      meta[0] = make_int2(0, 0);
      if (CIGAR) tab[0] = make_short2(0, 0);
    }
    fast_sync<G>();

    int final_flag = kStepDone;
    int parity = 0;  // buffer of the step parameters (every warp alike)
    while (true) {
      // ======================================== bookkeeping (first warp)
      FastStep st;
      parity ^= 1;
      if (wig == 0) {
        st.flag = kStepCells;
        st.used_lo = w_lo;
        st.used_hi = w_hi;
        if (done) {
          st.flag = kStepDone;
        } else if ((int64_t)p.g * s + 1 >= (int64_t)p.max_steps || s + 1 >= p.s_cap) {
          // the reference computes score g*s+1 next and stops there at the
          // step limit (wavefront/wavefront_unialign.c:102-107): the general
          // kernel reports that
          st.flag = kStepLeave;
        } else {
          ++s;
          cM = (cM + 1 == p.R) ? 0 : cM + 1;
          cI = (cI + 1 == p.RI) ? 0 : cI + 1;
          const int sMx = cM - p.x < 0 ? cM - p.x + p.R : cM - p.x;
          const int sMo = cM - p.oe < 0 ? cM - p.oe + p.R : cM - p.oe;
          const int sIe = cI - p.e < 0 ? cI - p.e + p.RI : cI - p.e;
          // input limits (wavefront/wavefront_compute.c:306-352; a score
          // below 0 is a null wavefront)
          const int2 kEmpty = make_int2(1, 0);
          const int2 eMx = s >= p.x ? meta[sMx] : kEmpty;
          const int2 eMo = s >= p.oe ? meta[sMo] : kEmpty;
          const int2 eI = s >= p.e ? meta[rowI + sIe] : kEmpty;
          const int2 eD = s >= p.e ? meta[rowD + sIe] : kEmpty;
          const bool vMx = eMx.x <= eMx.y, vMo = eMo.x <= eMo.y;
          const bool vI = eI.x <= eI.y, vD = eD.x <= eD.y;
          st.s = s;
          st.rMx = sMx * W + HALF;
          st.rMo = sMo * W + HALF;
          st.rI = (rowI + sIe) * W + HALF;
          st.rD = (rowD + sIe) * W + HALF;
          st.oM = cM * W + HALF;
          st.oI = (rowI + cI) * W + HALF;
          st.oD = (rowD + cI) * W + HALF;
          int16_t* const oM = rows + st.oM;
          int16_t* const oI = rows + st.oI;
          int16_t* const oD = rows + st.oD;
          const int2 oldM = meta[cM], oldI = meta[rowI + cI], oldD = meta[rowD + cI];
          st.oldM = oldM;
          st.oldI = oldI;
          st.oldD = oldD;
          if (!(vMx | vMo | vI | vD)) {
            // a null step (wavefront/wavefront_compute_affine.c:236-243): the
            // slots taken over become empty and all-NULL
            for (int k = oldM.x + lane; k <= oldM.y; k += 32) oM[k] = kNull16;
            for (int k = oldI.x + lane; k <= oldI.y; k += 32) oI[k] = kNull16;
            for (int k = oldD.x + lane; k <= oldD.y; k += 32) oD[k] = kNull16;
            __syncwarp();
            if (lane == 0) {
              meta[cM] = meta[rowI + cI] = meta[rowD + cI] = kEmpty;
              if (CIGAR) tab[s] = make_short2(1, 0);
            }
            __syncwarp();
            // more null steps than the scope: the end is unreachable
            // (wavefront/wavefront_extend.c:95-101), left to the general kernel
            st.flag = (++null_steps > p.R + 1) ? kStepLeave : kStepNull;
          } else {
            null_steps = 0;
            // output range: union of the inputs' (wavefront/wavefront_compute.c:40-87)
            int lo = INT_MAX, hi = INT_MIN;
            if (vMx) { lo = min(lo, eMx.x); hi = max(hi, eMx.y); }
            if (vMo) { lo = min(lo, eMo.x - 1); hi = max(hi, eMo.y + 1); }
            if (vI) { lo = min(lo, eI.x + 1); hi = max(hi, eI.y + 1); }
            if (vD) { lo = min(lo, eD.x - 1); hi = max(hi, eD.y - 1); }
            st.lo = lo;
            st.hi = hi;
            bt_used += hi - lo + 1;
            if (lo < 1 - HALF || hi > HALF - 2 ||  // wider than the rows
                (CIGAR && p.pair_cap > 0 && bt_used > p.pair_cap)) {  // over the pair's budget
              st.flag = kStepLeave;
            } else {
              w_lo = min(w_lo, lo);
              w_hi = max(w_hi, hi);
              st.used_lo = w_lo;
              st.used_hi = w_hi;
              // what the slots held outside [lo,hi] becomes NULL (disjoint
              // from the cells written next, and no input row is an output
              // row); in place, the slots are inputs too: after the cells
              if (!INPLACE) {
                if (oldM.x <= oldM.y && (oldM.x < lo || oldM.y > hi)) {
                  for (int k = oldM.x + lane; k <= min(oldM.y, lo - 1); k += 32) oM[k] = kNull16;
                  for (int k = max(oldM.x, hi + 1) + lane; k <= oldM.y; k += 32) oM[k] = kNull16;
                }
                if (oldI.x <= oldI.y && (oldI.x < lo || oldI.y > hi)) {
                  for (int k = oldI.x + lane; k <= min(oldI.y, lo - 1); k += 32) oI[k] = kNull16;
                  for (int k = max(oldI.x, hi + 1) + lane; k <= oldI.y; k += 32) oI[k] = kNull16;
                }
                if (oldD.x <= oldD.y && (oldD.x < lo || oldD.y > hi)) {
                  for (int k = oldD.x + lane; k <= min(oldD.y, lo - 1); k += 32) oD[k] = kNull16;
                  for (int k = max(oldD.x, hi + 1) + lane; k <= oldD.y; k += 32) oD[k] = kNull16;
                }
              }
              if (CIGAR && lane == 0) tab[s] = make_short2((short)lo, (short)hi);
            }
          }
        }
        if (G > 32 && lane == 0) info[parity] = st;
      }
      if (G > 32) {
        __syncthreads();  // A: the step's parameters and clears are visible
        if (wig != 0) st = info[parity];
      }
      if (st.flag >= kStepDone) {
        final_flag = st.flag;
        used_lo = st.used_lo;
        used_hi = st.used_hi;
        break;
      }
      if (st.flag == kStepNull) continue;

      // ======================================== the cells (every warp)
      const int lo = st.lo, hi = st.hi;
      const int16_t* const rMx = rows + st.rMx;
      const int16_t* const rMo = rows + st.rMo;
      const int16_t* const rI = rows + st.rI;
      const int16_t* const rD = rows + st.rD;
      int16_t* const oM = rows + st.oM;
      int16_t* const oI = rows + st.oI;
      int16_t* const oD = rows + st.oD;
      uint32_t* const crow = CIGAR ? codes + (int64_t)st.s * RW + t : nullptr;
      Mask mM = 0, mI = 0, mD = 0;  // bit j: cell lo+t+G*j in bounds
      uint32_t acc = 0;                 // 4-bit choice codes of 8 iterations
      int32_t n_mx = 0, n_mom = 0, n_mop = 0, n_ie = 0, n_de = 0;
      if (lo + t <= hi) {
        const int k = lo + t;
        n_mx = rMx[k]; n_mom = rMo[k - 1]; n_mop = rMo[k + 1]; n_ie = rI[k - 1]; n_de = rD[k + 1];
      }
      // the same trip count on every thread (cells past hi are skipped), so
      // the in-place ordering barrier below has every lane
      const int niter = (hi - lo + G) / G;
      for (int j = 0; j < niter; ++j) {
        const int k = lo + t + G * j;
        const int32_t mx = n_mx, mom = n_mom, mop = n_mop, ie = n_ie, de = n_de;
        const int kn = k + G;
        if (kn <= hi) {
          n_mx = rMx[kn]; n_mom = rMo[kn - 1]; n_mop = rMo[kn + 1]; n_ie = rI[kn - 1]; n_de = rD[kn + 1];
        }
        // In place, a step's output rows are its input rows: a lane's cell k
        // is read as k-1 or k+1 by its neighbours, whose reads of this
        // iteration's cells were all issued one iteration earlier; this
        // barrier orders the next iteration's reads before this one's writes.
        if (INPLACE) __syncwarp();
        if (k > hi) continue;
        // wavefront/wavefront_compute_affine.c:66-84
        const int32_t i1 = max(mom, ie) + 1;
        const int32_t d1 = max(mop, de);
        const int32_t mis = mx + 1;
        const int32_t best = max(d1, max(mis, i1));
        const int32_t v = best - k;
        const bool okM = (uint32_t)best <= (uint32_t)tlen && (uint32_t)v <= (uint32_t)plen;
        // extension (wavefront/wavefront_extend.c:86-121): the first 16-base
        // window without a branch (a NULL cell compares at 0,0 and is
        // discarded), further windows only for the rare long match
        const int ev = okM ? v : 0, eh = okM ? best : 0;
        const int lim = min(plen - ev, tlen - eh);
        const uint2 wa = QP[ev >> 4], wb = QT[eh >> 4];
        const uint32_t dx = __funnelshift_l(wa.x, wa.y, (uint32_t)ev << 1) ^
                            __funnelshift_l(wb.x, wb.y, (uint32_t)eh << 1);
        int L = dx ? (int)(__clz(dx) >> 1) : 16;
        if (okM && L == 16 && lim > 16) L = 16 + fast_lcp(QP, QT, ev + 16, eh + 16, lim - 16);
        const int32_t mext = okM ? best + min(L, lim) : kNull16;
        oM[k] = (int16_t)mext;
        oI[k] = (int16_t)i1;
        oD[k] = (int16_t)d1;
        const Mask bit = Mask(1) << j;
        if (okM) mM |= bit;
        if ((uint32_t)i1 <= (uint32_t)tlen) mI |= bit;
        if ((uint32_t)(d1 - k) <= (uint32_t)plen) mD |= bit;
        if (CIGAR) {
          // source of M: mismatch > deletion > insertion; gaps: extend >= open
          uint32_t c = (mis == best) ? 0u : (d1 == best ? 1u : 2u);
          c |= (uint32_t)(ie >= mom) << 2;
          c |= (uint32_t)(de >= mop) << 3;
          acc |= c << ((j & 7) << 2);
          if ((j & 7) == 7 || kn > hi) {
            crow[(j >> 3) * G] = acc;
            acc = 0;
          }
        }
      }
      if (INPLACE) {
        // what the slots held outside [lo,hi] (read as the neighbours of the
        // range's end cells) becomes NULL now
        __syncwarp();
        const int2 oM2 = st.oldM, oI2 = st.oldI, oD2 = st.oldD;
        if (oM2.x <= oM2.y && (oM2.x < lo || oM2.y > hi)) {
          for (int q = oM2.x + lane; q <= min(oM2.y, lo - 1); q += 32) oM[q] = kNull16;
          for (int q = max(oM2.x, hi + 1) + lane; q <= oM2.y; q += 32) oM[q] = kNull16;
        }
        if (oI2.x <= oI2.y && (oI2.x < lo || oI2.y > hi)) {
          for (int q = oI2.x + lane; q <= min(oI2.y, lo - 1); q += 32) oI[q] = kNull16;
          for (int q = max(oI2.x, hi + 1) + lane; q <= oI2.y; q += 32) oI[q] = kNull16;
        }
        if (oD2.x <= oD2.y && (oD2.x < lo || oD2.y > hi)) {
          for (int q = oD2.x + lane; q <= min(oD2.y, lo - 1); q += 32) oD[q] = kNull16;
          for (int q = max(oD2.x, hi + 1) + lane; q <= oD2.y; q += 32) oD[q] = kNull16;
        }
      }
      // first/last in-bounds cell per component (wavefront/wavefront_compute.c:
      // 579-613), as offsets G*j + t from lo
      auto first_of = [&](Mask m) -> int {
        if (!m) return INT_MAX;
        return G * (sizeof(Mask) == 8 ? __ffsll((long long)m) - 1 : __ffs((int)m) - 1) + t;
      };
      auto last_of = [&](Mask m) -> int {
        if (!m) return INT_MIN;
        return G * (sizeof(Mask) == 8 ? 63 - __clzll((long long)m) : 31 - __clz((int)m)) + t;
      };
      int fM = __reduce_min_sync(kFull, first_of(mM));
      int lM = __reduce_max_sync(kFull, last_of(mM));
      int fI = __reduce_min_sync(kFull, first_of(mI));
      int lI = __reduce_max_sync(kFull, last_of(mI));
      int fD = __reduce_min_sync(kFull, first_of(mD));
      int lD = __reduce_max_sync(kFull, last_of(mD));
      if (G > 32) {
        if (lane == 0) {
          int32_t* const pr = part + wig * 8;
          pr[0] = fM; pr[1] = lM; pr[2] = fI; pr[3] = lI; pr[4] = fD; pr[5] = lD;
        }
        __syncthreads();  // B: every cell and partial is written
      } else {
        __syncwarp();
      }
      // ======================================== trimming and the end test (first warp)
      if (wig == 0) {
        if (G > 32) {
          for (int w = 0; w < NW; ++w) {
            const int32_t* const q = part + w * 8;
            fM = min(fM, q[0]); lM = max(lM, q[1]);
            fI = min(fI, q[2]); lI = max(lI, q[3]);
            fD = min(fD, q[4]); lD = max(lD, q[5]);
          }
        }
        const int tloM = fM == INT_MAX ? 1 : lo + fM, thiM = fM == INT_MAX ? 0 : lo + lM;
        const int tloI = fI == INT_MAX ? 1 : lo + fI, thiI = fI == INT_MAX ? 0 : lo + lI;
        const int tloD = fD == INT_MAX ? 1 : lo + fD, thiD = fD == INT_MAX ? 0 : lo + lD;
        // M cells out of bounds are stored NULL.  I and D keep their values;
        // out-of-bounds ones at the trimmed ends become NULL, as the
        // reference's trim leaves them.  The trimmed-away ends are few cells.
        const int width = hi - lo + 1;
        const int nIL = fI == INT_MAX ? width : tloI - lo, nIR = fI == INT_MAX ? 0 : hi - thiI;
        const int nDL = fD == INT_MAX ? width : tloD - lo, nDR = fD == INT_MAX ? 0 : hi - thiD;
        const int nmax = max(max(nIL, nIR), max(nDL, nDR));
        bool fill = false;
        for (int q = lane; q < nmax; q += 32) {
          if (q < nIL) fill |= oI[lo + q] >= 0;
          if (q < nIR) fill |= oI[hi - q] >= 0;
          if (q < nDL) fill |= oD[lo + q] >= 0;
          if (q < nDR) fill |= oD[hi - q] >= 0;
        }
        if (__any_sync(kFull, fill)) {
          __syncwarp();
          for (int q = lane; q < nmax; q += 32) {
            if (q < nIL) oI[lo + q] = kNull16;
            if (q < nIR) oI[hi - q] = kNull16;
            if (q < nDL) oD[lo + q] = kNull16;
            if (q < nDR) oD[hi - q] = kNull16;
          }
          __syncwarp();
        }
        if (lane == 0) {
          meta[cM] = make_int2(tloM, thiM);
          meta[rowI + cI] = make_int2(tloI, thiI);
          meta[rowD + cI] = make_int2(tloD, thiD);
        }
        // termination on M[s] at k_end (wavefront/wavefront_termination.c:37-60)
        done = tloM <= k_end && k_end <= thiM && oM[k_end] >= tlen;
        __syncwarp();
      }
    }

    if (final_flag != kStepDone) {
      punt();
      fast_sync<G>();
      continue;
    }
    // the result (the first warp holds the score)
    if (wig == 0) {
      // classic score (wavefront/wavefront_compute.c:108-120) at WFA score
      // g*s, in the reference's wrapping int arithmetic
      const int S = p.g * s;
      const int score =
          p.match == 0 ? -S
                       : (int)((uint32_t)(-p.match) * ((uint32_t)plen + (uint32_t)tlen) - (uint32_t)S) / 2;
      if (!CIGAR) {
        if (lane == 0) {
          p.scores[pair] = score;
          p.status[pair] = kStCompleted;
          if (p.end_info) {
            p.end_info[3 * (int64_t)pair] = plen;
            p.end_info[3 * (int64_t)pair + 1] = tlen;
            p.end_info[3 * (int64_t)pair + 2] = S;
          }
        }
      } else {
        // ------------------------------------------------ back-trace
        // The rows' limits go to shared memory (the wavefront rows are no
        // longer needed; the next pair clears all of them).  Then walk the
        // choice codes from (s, k_end) in M to (0, 0), recording the
        // operations backwards with an 'E' at every M visit, and replay
        // forwards re-extending each M visit with the same LCP.
        short2* const stab = reinterpret_cast<short2*>(rows);
        for (int i = lane; i <= s; i += 32) stab[i] = tab[i];
        used_lo = -HALF;
        used_hi = HALF - 1;
        __syncwarp();
        auto code_at = [&](int ss, int kk, bool& bad) -> uint32_t {
          const short2 lh = stab[ss];
          const int r = kk - lh.x;
          if (r < 0 || kk > lh.y) {
            bad = true;
            return 0u;
          }
          const int jj = r / G, tt = r - jj * G;
          const uint32_t w = codes[(int64_t)ss * RW + (jj >> 3) * G + tt];
          return (w >> ((jj & 7) << 2)) & 15u;
        };
        if (!fast_backtrace<1>(p, pair, plen, tlen, s, k_end, score, S, QP, QT, items, lane,
                               code_at))
          punt();
      }
      if (G > 32 && lane == 0) {
        bcast[1] = used_lo;
        bcast[2] = used_hi;
      }
    }
    fast_sync<G>();
    if (G > 32) {
      used_lo = bcast[1];
      used_hi = bcast[2];
    }
  }
}

}  // namespace wf2g

// Kernel of the fast pass for (full CIGAR?, threads per pair, row width).
extern "C" void* wf2g_fast_kernel_ptr(int cigar, int group, int width) {
  using namespace wf2g;
#define WF2G_FAST_CASE(G, W) \
  if (group == G && width == W) \
    return cigar ? (void*)wfa_fast_kernel<true, G, W> : (void*)wfa_fast_kernel<false, G, W>;
  WF2G_FAST_CASE(32, 1024)
  WF2G_FAST_CASE(32, 1536)
  WF2G_FAST_CASE(32, 2048)
  WF2G_FAST_CASE(64, 1024)
  WF2G_FAST_CASE(64, 2048)
  WF2G_FAST_CASE(128, 1024)
  WF2G_FAST_CASE(128, 2048)
#undef WF2G_FAST_CASE
  return nullptr;
}

// wfa_fast2.cu -- the warp-per-pair fast kernel with two diagonals per lane.
//
// Same semantics and the same retry contract as wfa_fast.cu (a pair it cannot
// finish goes to the retry list, and the next pass takes it in full): exact
// gap-affine, end-to-end, A/C/G/T, scores divided by g = gcd(x, o+e, e).
// Served when the scaled x is even and the scaled e is odd (the default
// (4,6,2) scales to (2,4,1); with match < 0 the transformed penalties
// (2x-2m, 2o, 2e-m) of (4,6,2,-1) are (10,12,5)).
//
// Layout.  Each shared-memory row holds int16 offsets; the cells of the
// step at scaled score s are written as 16x2 words of diagonal pairs
// (a, a+1) with a = s (mod 2): the row of score s stores diagonal d at
// element W/2 + d - (s & 1).  Then, with x even and e odd:
//   * M[s-x] at (k, k+1) is one aligned word (same parity),
//   * I[s-e] at (k-1, k) and D[s-e] at (k+1, k+2) are one aligned word each
//     (opposite parity),
//   * M[s-(o+e)] at (k-1, k) and (k+1, k+2) are one word each when o+e is
//     odd, or two byte permutes of three words when it is even,
// so a lane computes two cells with 16x2 integer instructions (max.s16x2,
// add.s16x2, min.u16x2) from five or six 32-bit shared loads and writes
// three 32-bit words.  Rows are updated in place (max(x,o+e) M rows, e I and
// D rows): a lane's next words are loaded before the warp barrier that
// precedes its stores, and a store never overwrites a cell that a later
// lane or iteration still reads.
//
// Per cell, as the reference computes it (wavefront/wavefront_compute_affine.c:
// 66-84, wavefront/wavefront_extend.c:86-121): I = max(M[s-o-e][k-1],
// I[s-e][k-1]) + 1, D = max(M[s-o-e][k+1], D[s-e][k+1]), M = max(M[s-x][k]+1,
// I, D); M is NULL unless 0 <= h <= tlen and 0 <= h-k <= plen (unsigned
// compares on the clamped coordinates), else extended by the exact LCP.
// Trimming (wavefront/wavefront_compute.c:579-613) tests the end cells of
// each component's natural range (M: [lo, hi]; I: its sources' range shifted
// by +1; D: by -1) and scans only when one is out of bounds; I and D cells
// trimmed away become NULL.
//
// Choice codes: 4 bits per cell, 1 = the comparison failed: bit 0 "M from
// mismatch" (M[s-x]+1 >= max(I, D)), bit 1 "deletion over insertion"
// (D >= I), bit 2 "insertion extended" (I[s-e] >= M[s-o-e] at k-1), bit 3
// "deletion extended".  A lane writes one 16-bit entry per iteration (its
// two words' four cells).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "wfa_fast_common.cuh"
#include "wfa_kernels.cuh"

namespace wf2g {

__device__ __forceinline__ uint32_t vmax_s16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("max.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t vmin_s16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("min.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t vmin_u16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t vadd_s16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("add.s16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
// two int16 halves as one 16x2 word
__device__ __forceinline__ uint32_t pack16x2(int lo, int hi) {
  return ((uint32_t)lo & 0xFFFFu) | ((uint32_t)hi << 16);
}

// Kernel of the two-diagonals-per-lane fast pass.  CIGAR: full alignment or
// score only.  MOS: o+e (scaled) is even, so M[s-o-e] shares the output
// rows' parity.  W: elements per shared-memory row (diagonals
// [4-W/2, W/2-4] are computed).  D241: the scaled penalties are the
// default's (x, o+e, e) = (2, 4, 1), compiled in (rings of 4 M rows and 1 I
// and D row).  WFA: the wf-adaptive cut-off (wavefront/wavefront_heuristic.c:
// 229-289), the library's default heuristic.
template <bool CIGAR, bool MOS, int W, bool D241, bool WFA>
__global__ void __launch_bounds__(32) wfa_fast2_kernel(const FastParams p) {
  static_assert(!D241 || MOS, "o+e = 4 is even");
  const int X = D241 ? 2 : p.x, OE = D241 ? 4 : p.oe, E = D241 ? 1 : p.e;
  const int R = D241 ? 4 : p.R, RI = D241 ? 1 : p.RI;
  constexpr int HALF = W / 2;
  constexpr int JM = (HALF + 63) / 64;  // most iterations of a step (64 words each)
  constexpr int RW = JM * 16;           // 32-bit choice words per step (16 bits per lane per iteration)
  constexpr int WW = W / 2;             // words per row
  // a range with no cell: min/max over ranges need no validity tests
  constexpr int kBig = 1 << 20;
  // the step at which the first pass projects each pair's final score (the
  // projected score beyond which it leaves for the wider rows: p.probe_limit)
  constexpr int kProbe = 192;
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x;
  const int nrows = R + 2 * RI;
  // diagonals [-reach, reach] are computed (at most W/2 - 4)
  const int reach = min(p.reach, HALF - 4);
  int16_t* const rows = reinterpret_cast<int16_t*>(smem + p.rows_off);
  uint32_t* const rows32 = reinterpret_cast<uint32_t*>(smem + p.rows_off);
  // the two sequences' word pairs interleaved at the start of shared
  // memory: entry i (16 bytes) = {P pair i, T pair i}
  uint2* const QP = reinterpret_cast<uint2*>(smem);
  uint2* const QT = QP + 1;
  int2* const meta = reinterpret_cast<int2*>(smem + p.meta_off);
  // per ring slot, the cells its row may hold: its limits before a cut-off.
  // A cut only shrinks the limits; the cut cells stay readable as the
  // neighbours of the next steps' cells, as in the reference, where later
  // compute steps pad with NULL only beyond a wavefront's initialised window
  // (wavefront/wavefront_compute.c:498-527).  Without a cut-off it equals
  // the limits.
  int2* const win = meta + nrows;
  // per-warp slice: [choice words: s_cap rows of RW][row limits: s_cap short2][walk items]
  uint8_t* const slice = p.scratch + (int64_t)blockIdx.x * p.slice_bytes;
  uint32_t* const codes = reinterpret_cast<uint32_t*>(slice);
  short2* const tab = reinterpret_cast<short2*>(slice + (int64_t)p.s_cap * RW * 4);
  uint8_t* const items = slice + p.items_off;
  const int rowI = R, rowD = R + RI;

  for (int i = lane; i < nrows * WW; i += 32) rows32[i] = 0x80008000u;
  int used_lo = 0, used_hi = -1;  // words of every row the previous pair touched
  const int n_items = p.num_items_dev ? *p.num_items_dev : p.n_items;

  while (true) {
    // ---------------------------------------------------------- next pair
    int item = 0;
    if (lane == 0) item = atomicAdd(p.queue, 1);
    item = __shfl_sync(kFull, item, 0);
    if (item >= n_items) break;
    const int pair = p.items ? p.items[item] : item;
    const int plen = p.p_len[pair];
    const int tlen = p.t_len[pair];
    auto punt = [&]() {
      if (lane == 0) p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
    };

    // ---------------------------------------------------------- reset
    if (used_lo <= used_hi) {
      const int span = used_hi - used_lo + 1;
      for (int i = lane; i < nrows * span; i += 32) {
        const int r = i / span, j = i - r * span;
        rows32[r * WW + used_lo + j] = 0x80008000u;
      }
    }
    for (int r = lane; r < nrows; r += 32) meta[r] = win[r] = make_int2(kBig, -kBig);
    bool ok = fast_stage<32, 2>(p.seqs + p.p_off[pair], min(plen, p.max_len), QP, p.nq, lane);
    ok &= fast_stage<32, 2>(p.seqs + p.t_off[pair], min(tlen, p.max_len), QT, p.nq, lane);
    __syncwarp();
    const int k_end = tlen - plen;
    if (!ok || plen > p.max_len || tlen > p.max_len || k_end < -reach || k_end > reach) {
      punt();
      used_lo = 0;
      used_hi = -1;
      __syncwarp();
      continue;
    }

    // ---------------------------------------------------------- score 0
    // M[0][0] = 0, extended at once (wavefront/wavefront_aligner.c:311-382)
    const int L0 = fast_lcp<2>(QP, QT, 0, 0, min(plen, tlen));
    int s = 0;           // scaled score of the last computed wavefront
    int cM = 0, cI = 0;  // its ring slots
    int null_steps = 0;
    int64_t bt_used = 0;     // choice codes of the pair: the general kernel's byte count
    int w_lo = 0, w_hi = 0;  // diagonals touched
    bool done = (plen == tlen) && (L0 >= tlen);
    int steps_wait = WFA ? p.h_steps : 0;  // steps to the next cut-off
    if (WFA && !done) {
      // the cut-off of M[0]: one cell, never cut; it counts toward the wait
      --steps_wait;
      if (steps_wait <= 0 && 1 >= p.h_min_len) steps_wait = p.h_steps;
    }
    if (lane == 0) {
      rows[HALF] = (int16_t)L0;  // row 0 (slot 0 of M, parity 0), diagonal 0
      meta[0] = win[0] = make_int2(0, 0);
      if (CIGAR) tab[0] = make_short2(0, 0);
    }
    __syncwarp();
    const uint32_t plen2 = pack16x2(plen, plen), tlen2 = pack16x2(tlen, tlen);

    // the last scaled score to compute: step s -> s+1 needs g*s + 1 <
    // max_steps (the reference computes score g*s+1 next and stops there at
    // the step limit) and s + 1 < s_cap
    const int64_t s_steps = p.max_steps >= 2 ? ((int64_t)p.max_steps - 2) / p.g + 1 : -1;
    const int s_lim = (int)(s_steps < p.s_cap - 1 ? s_steps : (int64_t)(p.s_cap - 1));
    bool leave = false;
    while (!done) {
      if (s + 1 > s_lim) {
        // the reference computes score g*s+1 next and stops there at the
        // step limit (wavefront/wavefront_unialign.c:102-107): the general
        // kernel reports that
        leave = true;
        break;
      }
      ++s;
      const int par = s & 1;
      cM = (cM + 1 == R) ? 0 : cM + 1;
      cI = (cI + 1 == RI) ? 0 : cI + 1;
      const int sMx = cM - X < 0 ? cM - X + R : cM - X;
      const int sMo = cM - OE < 0 ? cM - OE + R : cM - OE;
      const int sIe = cI - E < 0 ? cI - E + RI : cI - E;
      // input limits (wavefront/wavefront_compute.c:306-352).  A score below
      // 0 is a null wavefront: its slot (s - d + R >= s for d <= R) has not
      // been written for this pair yet and still holds the empty range.
      const int2 kEmpty = make_int2(kBig, -kBig);
      const int2 eMx = meta[sMx];
      const int2 eMo = meta[sMo];
      const int2 eI = meta[rowI + sIe];
      const int2 eD = meta[rowD + sIe];
      // element of diagonal 0 in the output slots (this step's parity), and
      // in the same slots' previous contents (scores s-R and s-RI)
      const int bM = cM * W + HALF - par;
      const int bI = (rowI + cI) * W + HALF - par;
      const int bD = (rowD + cI) * W + HALF - par;
      const int obM = cM * W + HALF - ((s - R) & 1);
      const int obI = (rowI + cI) * W + HALF - ((s - RI) & 1);
      const int obD = (rowD + cI) * W + HALF - ((s - RI) & 1);
      // the output slots' previous contents (the inputs themselves when the
      // ring is exactly as long as their distance)
      const int2 oldM = WFA ? win[cM] : (R == OE) ? eMo : meta[cM];
      const int2 oldI = WFA ? win[rowI + cI] : (RI == E) ? eI : meta[rowI + cI];
      const int2 oldD = WFA ? win[rowD + cI] : (RI == E) ? eD : meta[rowD + cI];
      // output range: union of the inputs' (wavefront/wavefront_compute.c:40-87)
      const int lo = min(min(eMx.x, eMo.x - 1), min(eI.x + 1, eD.x - 1));
      const int hi = max(max(eMx.y, eMo.y + 1), max(eI.y + 1, eD.y - 1));
      if (lo > hi) {
        // a null step (wavefront/wavefront_compute_affine.c:236-243): the
        // slots taken over become empty and all-NULL
        for (int k = oldM.x + lane; k <= oldM.y; k += 32) rows[obM + k] = kNull16;
        for (int k = oldI.x + lane; k <= oldI.y; k += 32) rows[obI + k] = kNull16;
        for (int k = oldD.x + lane; k <= oldD.y; k += 32) rows[obD + k] = kNull16;
        __syncwarp();
        if (lane == 0) {
          meta[cM] = meta[rowI + cI] = meta[rowD + cI] = kEmpty;
          win[cM] = win[rowI + cI] = win[rowD + cI] = kEmpty;
          if (CIGAR) tab[s] = make_short2(1, 0);
        }
        __syncwarp();
        // more null steps than the scope: the end is unreachable
        // (wavefront/wavefront_extend.c:95-101), left to the general kernel
        if (++null_steps > R + 1) {
          leave = true;
          break;
        }
        continue;
      }
      null_steps = 0;
      bt_used += hi - lo + 1;
      if (lo < -reach || hi > reach ||  // wider than the rows
          (CIGAR && p.pair_cap > 0 && bt_used > p.pair_cap)) {  // over the pair's budget
        leave = true;
        break;
      }
      w_lo = min(w_lo, lo);
      w_hi = max(w_hi, hi);
      // (every lane stores the same value: no divergent branch per step)
      if (CIGAR) tab[s] = make_short2((short)lo, (short)hi);
      // the natural ranges of I (sources at k-1) and D (sources at k+1): the
      // cells of [lo, hi] outside them are computed from NULL or NULL-ish
      // (negative) inputs only, so they come out negative, out of bounds
      // (under a cut-off the sources' windows, clamped to [lo, hi])
      int iLo, iHi, dLo, dHi;
      if (WFA) {
        const int2 wMo = win[sMo], wI = win[rowI + sIe], wD = win[rowD + sIe];
        iLo = max(lo, min(wMo.x, wI.x) + 1);
        iHi = min(hi, max(wMo.y, wI.y) + 1);
        dLo = max(lo, min(wMo.x, wD.x) - 1);
        dHi = min(hi, max(wMo.y, wD.y) - 1);
      } else {
        iLo = min(eMo.x, eI.x) + 1;
        iHi = max(eMo.y, eI.y) + 1;
        dLo = min(eMo.x, eD.x) - 1;
        dHi = max(eMo.y, eD.y) - 1;
      }

      // ======================================== the cells
      // pairs (a0 + 2q, a0 + 2q + 1), a0 = s (mod 2), q < nq; lane q % 32
      const int a0 = lo - ((lo - par) & 1);
      const int nq = ((hi - a0) >> 1) + 1;
      // word of pair 0 in a row of this step's parity (element W/2 + a0 - par
      // is even); the other parity's (k-1, k) word is hb + par - 1 and its
      // (k+1, k+2) word hb + par
      const int hb = (HALF + a0 - par) >> 1;
      const uint32_t* const wMx = rows32 + sMx * WW + hb;
      const uint32_t* const wMo = rows32 + sMo * WW + (MOS ? hb : hb + par - 1);
      const uint32_t* const wI = rows32 + (rowI + sIe) * WW + hb + par - 1;
      const uint32_t* const wD = rows32 + (rowD + sIe) * WW + hb + par;
      uint32_t* const oM = rows32 + cM * WW + hb;
      uint32_t* const oI = rows32 + (rowI + cI) * WW + hb;
      uint32_t* const oD = rows32 + (rowD + cI) * WW + hb;
      // choice codes: a 16-bit entry per lane and iteration
      uint16_t* const crow = CIGAR ? reinterpret_cast<uint16_t*>(codes + (int64_t)s * RW) + lane : nullptr;
      // The inputs of one word (two cells): M[s-x] at (k, k+1), M[s-o-e] at
      // (k-1, k) and (k+1, k+2), I[s-e] at (k-1, k), D[s-e] at (k+1, k+2).
      struct In { uint32_t x, mm, mp, i, d; };
      auto load = [&](int q) -> In {
        In r;
        r.x = wMx[q];
        if (MOS) {
          const uint32_t w0 = wMo[q - 1], w1 = wMo[q], w2 = wMo[q + 1];
          r.mm = __byte_perm(w0, w1, 0x5432);  // (k-1, k)
          r.mp = __byte_perm(w1, w2, 0x5432);  // (k+1, k+2)
        } else {
          r.mm = wMo[q];
          r.mp = wMo[q + 1];
        }
        r.i = wI[q];
        r.d = wD[q];
        return r;
      };
      const char* const qs = reinterpret_cast<const char*>(smem);
      // One word: the cells (k, k+1), k = a0 + 2q, with kvp = (k + plen,
      // k + 1 + plen) and negk = (-k, -k-1) as 16x2.  Stores the word's M, I and D and returns
      // its choice codes (low half: cell k, high half: cell k+1).
      auto cells = [&](int q, const In& in, uint32_t kvp, uint32_t negk) -> uint32_t {
        const uint32_t moi = vmax_s16x2(in.mm, in.i);        // max(M[s-o-e][k-1], I[s-e][k-1])
        const uint32_t i1 = vadd_s16x2(moi, 0x00010001u);
        const uint32_t d1 = vmax_s16x2(in.mp, in.d);         // max(M[s-o-e][k+1], D[s-e][k+1])
        const uint32_t mis = vadd_s16x2(in.x, 0x00010001u);
        const uint32_t gap = vmax_s16x2(d1, i1);
        const uint32_t best = vmax_s16x2(mis, gap);
        // h = best, v = best - k, clamped into the sequences; a clamp that
        // changed either marks the cell out of bounds
        const uint32_t vv = vadd_s16x2(best, negk);
        const uint32_t hc = vmin_u16x2(best, tlen2), vc = vmin_u16x2(vv, plen2);
        const uint32_t oob = (hc ^ best) | (vc ^ vv);
        // first 16-base windows of both cells: the 16-byte entries at
        // (v >> 4) * 16 = v & ~15 (P) and h & ~15 (+8: T), and funnel
        // shifts (only their low 5 bits count)
        const uint2 pa0 = *reinterpret_cast<const uint2*>(qs + (vc & 0xFFF0u));
        const uint2 pa1 = *reinterpret_cast<const uint2*>(qs + ((vc >> 16) & 0xFFF0u));
        const uint2 ta0 = *reinterpret_cast<const uint2*>(qs + 8 + (hc & 0xFFF0u));
        const uint2 ta1 = *reinterpret_cast<const uint2*>(qs + 8 + ((hc >> 16) & 0xFFF0u));
        const uint32_t x0 = __funnelshift_l(pa0.x, pa0.y, vc << 1) ^
                            __funnelshift_l(ta0.x, ta0.y, hc << 1);
        const uint32_t x1 = __funnelshift_l(pa1.x, pa1.y, vc >> 15) ^
                            __funnelshift_l(ta1.x, ta1.y, hc >> 15);
        int L0c = __clz(x0) >> 1, L1c = __clz(x1) >> 1;
        if ((x0 == 0) | (x1 == 0)) {
          // a whole window matched: further windows, for cells in bounds
          const int ev0 = vc & 0xFFFF, ev1 = vc >> 16, eh0 = hc & 0xFFFF, eh1 = hc >> 16;
          if (x0 == 0 && (oob & 0xFFFFu) == 0) {
            const int lim = min(plen - ev0, tlen - eh0);
            if (lim > 16) L0c = 16 + fast_lcp<2>(QP, QT, ev0 + 16, eh0 + 16, lim - 16);
          }
          if (x1 == 0 && (oob >> 16) == 0) {
            const int lim = min(plen - ev1, tlen - eh1);
            if (lim > 16) L1c = 16 + fast_lcp<2>(QP, QT, ev1 + 16, eh1 + 16, lim - 16);
          }
        }
        // extended offset, capped at min(plen + k, tlen) (the end of the
        // shorter rest); NULL out of bounds (exactly: the cap can be -1 on
        // diagonal -plen-1, where a set sign bit alone would leave -1)
        const uint32_t capv = vmin_s16x2(kvp, tlen2);
        const uint32_t mext = vmin_s16x2(vadd_s16x2(best, (uint32_t)L0c | ((uint32_t)L1c << 16)), capv);
        const uint32_t nullm = vmin_u16x2(oob, 0x00010001u) * 0xFFFFu;
        oM[q] = (mext & ~nullm) | (0x80008000u & nullm);
        oI[q] = i1;
        oD[q] = d1;
        if (!CIGAR) return 0u;
        const uint32_t f0 = vmin_u16x2(best ^ mis, 0x00010001u);
        const uint32_t f1 = vmin_u16x2(gap ^ d1, 0x00010001u);
        const uint32_t f2 = vmin_u16x2(moi ^ in.i, 0x00010001u);
        const uint32_t f3 = vmin_u16x2(d1 ^ in.d, 0x00010001u);
        return f0 | (f1 << 1) | (f2 << 2) | (f3 << 3);
      };
      // Lane t takes words t + 32m, m = 0 .. mlast; two per iteration (m =
      // 2j and 2j+1), two independent chains.  Choice codes: per iteration a
      // 16-bit entry per lane, nibbles [word 2j low cell, word 2j+1 low
      // cell, word 2j high cell, word 2j+1 high cell].
      const int mlast = (nq - 1) >> 5;
      const int niter = (mlast >> 1) + 1;
      In n0{}, n1{};
      if (lane < nq) n0 = load(lane);
      if (lane + 32 < nq) n1 = load(lane + 32);
      uint32_t kvp0 = pack16x2(a0 + 2 * lane + plen, a0 + 2 * lane + 1 + plen);
      uint32_t negk0 = pack16x2(-a0 - 2 * lane, -a0 - 2 * lane - 1);
      for (int j = 0; j < niter; ++j) {
        const In c0 = n0, c1 = n1;
        const int q0 = lane + 64 * j, q1 = q0 + 32;
        if (q0 + 64 < nq) n0 = load(q0 + 64);
        if (q1 + 64 < nq) n1 = load(q1 + 64);
        // in place: this iteration's stores overwrite cells that the next
        // iteration's loads (just issued) and this iteration's neighbours
        // read; the barrier orders every lane's loads before the stores
        __syncwarp();
        uint32_t code = 0;
        if (q0 < nq) code = cells(q0, c0, kvp0, negk0);
        if (q1 < nq)
          code |= cells(q1, c1, vadd_s16x2(kvp0, 0x00400040u), vadd_s16x2(negk0, 0xFFC0FFC0u)) << 4;
        if (CIGAR) crow[j * 32] = (uint16_t)__byte_perm(code, 0u, 0x4420u);
        kvp0 = vadd_s16x2(kvp0, 0x00800080u);
        negk0 = vadd_s16x2(negk0, 0xFF80FF80u);
      }
      __syncwarp();
      // Cells written outside [lo, hi] (the first pair's low cell, the last
      // pair's high cell) become NULL, and so do the slots' previous contents
      // outside the written cells [a0, aL].  A previous content at score s'
      // sits one element off when s' has the other parity: in this step's
      // diagonals it spans [x + sh, y + sh], sh = (s & 1) - (s' & 1).
      const int aL = a0 + 2 * nq - 1;
      if (a0 < lo) rows[bM + a0] = rows[bI + a0] = rows[bD + a0] = kNull16;
      if (aL > hi) rows[bM + aL] = rows[bI + aL] = rows[bD + aL] = kNull16;
      {
        const int shM = par - ((s - R) & 1), shI = par - ((s - RI) & 1);
        // (with a ring exactly o+e long the old M row is M[s-o-e], whose
        // range the written span covers)
        const bool cM_ = (WFA || R != OE) && oldM.x <= oldM.y && (oldM.x + shM < a0 || oldM.y + shM > aL);
        const bool cI_ = oldI.x <= oldI.y && (oldI.x + shI < a0 || oldI.y + shI > aL);
        const bool cD_ = oldD.x <= oldD.y && (oldD.x + shI < a0 || oldD.y + shI > aL);
        if (cM_ | cI_ | cD_) {
          auto clear_outside = [&](int base, int x, int y) {  // diagonals [x, y] at base, minus [a0, aL]
            for (int k = x + lane; k <= min(y, a0 - 1); k += 32) rows[base + k] = kNull16;
            for (int k = max(x, aL + 1) + lane; k <= y; k += 32) rows[base + k] = kNull16;
          };
          if (cM_) clear_outside(bM, oldM.x + shM, oldM.y + shM);
          if (cI_) clear_outside(bI, oldI.x + shI, oldI.y + shI);
          if (cD_) clear_outside(bD, oldD.x + shI, oldD.y + shI);
        }
      }
      __syncwarp();
      // first/last in-bounds cell per component (wavefront/wavefront_compute.c:
      // 579-613): M is not NULL (over [lo, hi]); I has h <= tlen and D has
      // h - k <= plen (over their natural ranges).  Lanes 0-5 test the six
      // end cells; only a component with an end out of bounds is scanned.
      auto inb = [&](int comp, int k) -> bool {
        const int v = rows[(comp == 0 ? bM : comp == 1 ? bI : bD) + k];
        return comp == 0 ? v != kNull16
                         : comp == 1 ? (uint32_t)v <= (uint32_t)tlen : (uint32_t)(v - k) <= (uint32_t)plen;
      };
      const bool iE = iLo > iHi, dE = dLo > dHi;  // no I (D) cell has a source
      // (lanes 6-31 repeat lane 4's and 5's test, so no lane branches)
      const int comp = min(lane >> 1, 2), hiend = lane & 1;
      const int kend = comp == 0 ? (hiend ? hi : lo) : comp == 1 ? (hiend ? iHi : iLo) : (hiend ? dHi : dLo);
      const bool endok = (comp == 1 && iE) || (comp == 2 && dE) || inb(comp, kend);
      const uint32_t ends = __ballot_sync(kFull, endok) & 0x3Fu;
      int fM = lo, lM = hi;
      int fI = iE ? INT_MAX : iLo, lI = iE ? INT_MIN : iHi;
      int fD = dE ? INT_MAX : dLo, lD = dE ? INT_MIN : dHi;
      if (ends != 0x3Fu) {
        auto first_in = [&](int comp, int a, int b) -> int {
          for (int c = a; c <= b; c += 32) {
            const int k = c + lane;
            const uint32_t m = __ballot_sync(kFull, k <= b && inb(comp, k));
            if (m) return c + __ffs(m) - 1;
          }
          return INT_MAX;
        };
        auto last_in = [&](int comp, int a, int b) -> int {
          for (int c = b; c >= a; c -= 32) {
            const int k = c - lane;
            const uint32_t m = __ballot_sync(kFull, k >= a && inb(comp, k));
            if (m) return c - (__ffs(m) - 1);
          }
          return INT_MIN;
        };
        if ((ends & 3u) != 3u) {
          fM = first_in(0, lo, hi);
          lM = fM == INT_MAX ? INT_MIN : last_in(0, lo, hi);
        }
        // I and D cells of the natural ranges trimmed away become NULL (M out
        // of bounds is NULL already)
        if (((ends >> 2) & 3u) != 3u) {
          fI = first_in(1, iLo, iHi);
          lI = fI == INT_MAX ? INT_MIN : last_in(1, iLo, iHi);
          const int nL = fI == INT_MAX ? iHi - iLo + 1 : fI - iLo, nR = fI == INT_MAX ? 0 : iHi - lI;
          for (int q = lane; q < nL; q += 32) rows[bI + iLo + q] = kNull16;
          for (int q = lane; q < nR; q += 32) rows[bI + iHi - q] = kNull16;
        }
        if (((ends >> 4) & 3u) != 3u) {
          fD = first_in(2, dLo, dHi);
          lD = fD == INT_MAX ? INT_MIN : last_in(2, dLo, dHi);
          const int nL = fD == INT_MAX ? dHi - dLo + 1 : fD - dLo, nR = fD == INT_MAX ? 0 : dHi - lD;
          for (int q = lane; q < nL; q += 32) rows[bD + dLo + q] = kNull16;
          for (int q = lane; q < nR; q += 32) rows[bD + dHi - q] = kNull16;
        }
      }
      int2 tM = fM == INT_MAX ? kEmpty : make_int2(fM, lM);
      int2 tI = fI == INT_MAX ? kEmpty : make_int2(fI, lI);
      int2 tD = fD == INT_MAX ? kEmpty : make_int2(fD, lD);
      // termination on M[s] at k_end (wavefront/wavefront_termination.c:37-60)
      done = tM.x <= k_end && k_end <= tM.y && rows[bM + k_end] >= tlen;
      if (WFA) {
        win[cM] = tM;
        win[rowI + cI] = tI;
        win[rowD + cI] = tD;
      }
      if (!WFA && W == 1024 && s == kProbe && !done && tM.x <= tM.y) {
        // a pair whose progress so far (the furthest antidiagonal h + v)
        // projects a final scaled score beyond these rows' reach (the range
        // grows a diagonal per scaled step: +-508 is reached near 500)
        // leaves now for the wider pass instead of at the edge; a scheduling
        // choice only (the wider pass recomputes it in full).  Not under the
        // cut-off, which keeps the range narrow and the projection wrong.
        int prog = 0;
        for (int k = tM.x + lane; k <= tM.y; k += 32) {
          const int off = rows[bM + k];
          if (off >= 0) prog = max(prog, 2 * off - k);
        }
        prog = __reduce_max_sync(kFull, prog);
        if ((int64_t)kProbe * (plen + tlen) > (int64_t)p.probe_limit * max(prog, 1)) {
          leave = true;
          __syncwarp();
          break;
        }
      }
      const int2 winM = tM, winI = tI, winD = tD;  // the windows, before a cut
      if (WFA && !done && tM.x <= tM.y) {
        // wf-adaptive cut-off of the extended M[s] (wavefront/wavefront_
        // heuristic.c:229-289, dispatch :506-563): cells further from the end
        // than the closest by more than max_distance_threshold are cut from
        // both ends, keeping the end diagonal's side; I and D take the
        // intersection of limits
        --steps_wait;
        if (steps_wait <= 0 && tM.y - tM.x + 1 >= p.h_min_len) {
          auto dist = [&](int k) -> int {
            const int off = rows[bM + k];
            return off < 0 ? (1 << 30) : max(plen - (off - k), tlen - off);
          };
          int dmin = max(plen, tlen);
          for (int k = tM.x + lane; k <= tM.y; k += 32) dmin = min(dmin, dist(k));
          dmin = __reduce_min_sync(kFull, dmin);
          const int top = min(k_end, tM.y);
          int nlo = max(tM.x, top);
          for (int c = tM.x; c < top; c += 32) {
            const int k = c + lane;
            const uint32_t m = __ballot_sync(kFull, k < top && dist(k) - dmin <= p.h_max_dist);
            if (m) {
              nlo = c + __ffs(m) - 1;
              break;
            }
          }
          const int bot = max(k_end, nlo);
          int nhi = min(tM.y, bot);
          for (int c = tM.y; c > bot; c -= 32) {
            const int k = c - lane;
            const uint32_t m = __ballot_sync(kFull, k > bot && dist(k) - dmin <= p.h_max_dist);
            if (m) {
              nhi = c - (__ffs(m) - 1);
              break;
            }
          }
          steps_wait = p.h_steps;
          if (nlo != tM.x || nhi != tM.y) {
            tM = make_int2(nlo, nhi);
            tI = make_int2(max(tI.x, nlo), min(tI.y, nhi));
            tD = make_int2(max(tD.x, nlo), min(tD.y, nhi));
            // a row the cut empties reads as NULL everywhere (its window too)
            if (tM.x > tM.y) {
              for (int k = winM.x + lane; k <= winM.y; k += 32) rows[bM + k] = kNull16;
              tM = kEmpty;
              win[cM] = kEmpty;
            }
            if (tI.x > tI.y) {
              for (int k = winI.x + lane; k <= winI.y; k += 32) rows[bI + k] = kNull16;
              tI = kEmpty;
              win[rowI + cI] = kEmpty;
            }
            if (tD.x > tD.y) {
              for (int k = winD.x + lane; k <= winD.y; k += 32) rows[bD + k] = kNull16;
              tD = kEmpty;
              win[rowD + cI] = kEmpty;
            }
          }
        }
      }
      meta[cM] = tM;
      meta[rowI + cI] = tI;
      meta[rowD + cI] = tD;
      __syncwarp();
    }
    // words touched by this pair: elements [W/2 + w_lo - 4, W/2 + w_hi + 3]
    used_lo = (HALF + w_lo - 4) >> 1;
    used_hi = (HALF + w_hi + 3) >> 1;

    if (leave) {
      punt();
      __syncwarp();
      continue;
    }
    // the result: the classic score (wavefront/wavefront_compute.c:108-120)
    // at WFA score g*s, in the reference's wrapping int arithmetic
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
      // The rows' limits go to shared memory (the rows are no longer needed;
      // the next pair clears all of them), then the walk and the replay.
      short2* const stab = reinterpret_cast<short2*>(rows);
      for (int i = lane; i <= s; i += 32) stab[i] = tab[i];
      used_lo = 0;
      used_hi = WW - 1;
      __syncwarp();
      auto code_at = [&](int ss, int kk, bool& bad) -> uint32_t {
        const short2 lh = stab[ss];
        if (kk < lh.x || kk > lh.y) {
          bad = true;
          return 0u;
        }
        const int a0s = lh.x - ((lh.x - (ss & 1)) & 1);
        const int r = kk - a0s, q = r >> 1;
        const uint32_t w =
            reinterpret_cast<const uint16_t*>(codes + (int64_t)ss * RW)[(q >> 6) * 32 + (q & 31)];
        const uint32_t z = (w >> (((r & 1) << 3) + (((q >> 5) & 1) << 2))) & 15u;
        // to the walk's code: source of M (0 mismatch, 1 deletion, 2
        // insertion), bit 2 insertion extended, bit 3 deletion extended
        return (!(z & 1u) ? 0u : (!(z & 2u) ? 1u : 2u)) | (~z & 12u);
      };
      if (!fast_backtrace<2>(p, pair, plen, tlen, s, k_end, score, S, QP, QT, items, lane, code_at))
        punt();
    }
    __syncwarp();
  }
}

}  // namespace wf2g

// Kernel of the two-diagonals-per-lane pass for (full CIGAR?, o+e even?, row
// width, default scaled penalties (2, 4, 1)?, wf-adaptive cut-off?).  The
// cut-off is compiled for the default penalties only, and not for
// score-only rows of 1536 diagonals: that instance returned worse scores
// than the oracle on GB300 for pairs the 1024-, 2048-row and full-CIGAR
// 1536-row instances (and a CPU emulation of the kernel at every width) get
// right, and the difference went away when unrelated code was added, so the
// score-only wf-adaptive second pass takes rows of 2048 instead.
extern "C" void* wf2g_fast2_kernel_ptr(int cigar, int mos, int width, int d241, int wfa) {
  using namespace wf2g;
#define WF2G_FAST2_CASE(W)                                                                        \
  if (width == W) {                                                                               \
    if (wfa) {                                                                                    \
      if (!d241 || (W == 1536 && !cigar)) return nullptr;                                         \
      return cigar ? (void*)wfa_fast2_kernel<true, true, W, true, true>                           \
                   : (void*)wfa_fast2_kernel<false, true, W == 1536 ? 2048 : W, true, true>;      \
    }                                                                                             \
    if (d241) return cigar ? (void*)wfa_fast2_kernel<true, true, W, true, false>                  \
                           : (void*)wfa_fast2_kernel<false, true, W, true, false>;                \
    if (mos) return cigar ? (void*)wfa_fast2_kernel<true, true, W, false, false>                  \
                          : (void*)wfa_fast2_kernel<false, true, W, false, false>;                \
    return cigar ? (void*)wfa_fast2_kernel<true, false, W, false, false>                          \
                 : (void*)wfa_fast2_kernel<false, false, W, false, false>;                        \
  }
  WF2G_FAST2_CASE(1024)
  WF2G_FAST2_CASE(1536)
  WF2G_FAST2_CASE(2048)
#undef WF2G_FAST2_CASE
  return nullptr;
}

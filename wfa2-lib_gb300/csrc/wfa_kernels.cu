// wfa_kernels.cu -- sm_103a kernels of the GB300 wavefront aligner.
//
// Semantics follow smarco/WFA2-lib's exact unidirectional WFA (end-to-end):
//   compute   wavefront/wavefront_compute_affine.c:44-86,
//             wavefront/wavefront_compute_affine2p.c:45-106
//   limits    wavefront/wavefront_compute.c:40-87 (output range = union of inputs)
//   trim      wavefront/wavefront_compute.c:579-613 (ends only; interior kept)
//   extend    wavefront/wavefront_extend.c:86-121 (exact LCP per diagonal)
//   terminate wavefront/wavefront_termination.c:37-60
//   loop      wavefront/wavefront_unialign.c:242-273, limits :98-143
//   backtrace wavefront/wavefront_backtrace.c:320-529 -- reproduced from
//             per-cell choice bits: ties resolve exactly as the reference's
//             (offset<<4|type) maximum does: mismatch > D2 > D1 > I2 > I1,
//             extension > opening (wavefront/wavefront_backtrace.c:49-59).
//
// GPU design: one warp per pair, lanes striped over diagonals k; wavefront
// rows live in a (k mod WCAP) ring; a row is NULL outside its trimmed range
// (the reference's NULL padding, wavefront/wavefront_compute.c:498-575), so
// reads need no bounds checks.  Offsets are int32 with any negative == NULL.
#include <cuda_runtime.h>

#include <cstdint>

#include "wfa_kernels.cuh"

namespace wf2g {

// NULL as stored in a ring of OffT (int16 rings serve sequences < 32000).
template <typename OffT>
__device__ __forceinline__ OffT null_of() {
  return sizeof(OffT) == 2 ? (OffT)(-32768) : (OffT)kNull;
}
// Stores an offset; every negative value is NULL.
template <typename OffT>
__device__ __forceinline__ void put(OffT* row, int idx, int32_t v) {
  row[idx] = v < 0 ? null_of<OffT>() : (OffT)v;
}

__device__ __forceinline__ int ring_mod_back(int cur, int d, int R) {
  // slot of score (s-d) when slot of s is cur, 0 <= d < R
  const int t = cur - d;
  return t < 0 ? t + R : t;
}

// ---------------------------------------------------------------- sequences
// 2-bit: base i of a sequence at bits [63-2(i%32), 62-2(i%32)] of word i/32.
__device__ __forceinline__ uint64_t window2(const uint64_t* W, int pos) {
  const int w = pos >> 5;
  const int sh = (pos & 31) << 1;
  uint64_t x = W[w];
  if (sh) x = (x << sh) | (W[w + 1] >> (64 - sh));
  return x;
}
// 8-bit: byte i at bits [63-8(i%8), 56-8(i%8)] of word i/8.
__device__ __forceinline__ uint64_t window8(const uint64_t* W, int pos) {
  const int w = pos >> 3;
  const int sh = (pos & 7) << 3;
  uint64_t x = W[w];
  if (sh) x = (x << sh) | (W[w + 1] >> (64 - sh));
  return x;
}

// Longest common prefix of P[v..] and T[h..], at most lim characters:
// 64-bit XOR + count-leading-zeros per block (wavefront/wavefront_extend_kernels.c:68-92).
template <int ENC>
__device__ __forceinline__ int lcp(const uint64_t* P, const uint64_t* T, int v, int h, int lim) {
  constexpr int kPer = (ENC == 2) ? 32 : 8;
  constexpr int kShift = (ENC == 2) ? 1 : 3;
  int L = 0;
  while (L < lim) {
    const uint64_t a = (ENC == 2) ? window2(P, v + L) : window8(P, v + L);
    const uint64_t b = (ENC == 2) ? window2(T, h + L) : window8(T, h + L);
    const uint64_t d = a ^ b;
    if (d) {
      L += __clzll(d) >> kShift;
      break;
    }
    L += kPer;
  }
  return L < lim ? L : lim;
}

// Stages one sequence into W (warp-cooperative).  Returns false if ENC==2 and
// the sequence holds a byte outside {A,C,G,T}.
template <int ENC>
__device__ bool stage_sequence(const uint8_t* __restrict__ src, int len, uint64_t* W, int nwords,
                               int lane) {
  bool ok = true;
  if (ENC == 2) {
    const int nblk = (len + 31) >> 5;
    for (int b = 0; b < nblk; ++b) {
      const int i = (b << 5) + lane;
      uint32_t code = 0;
      if (i < len) {
        const uint8_t c = src[i];
        const bool valid = (c == 'A') | (c == 'C') | (c == 'G') | (c == 'T');
        ok &= valid;
        code = (c >> 1) & 3u;  // A0 C1 T2 G3 -- a bijection on ACGT
      }
      const uint32_t hi = __reduce_or_sync(kFull, lane < 16 ? code << (30 - 2 * lane) : 0u);
      const uint32_t lo = __reduce_or_sync(kFull, lane >= 16 ? code << (30 - 2 * (lane - 16)) : 0u);
      if (lane == 0) W[b] = ((uint64_t)hi << 32) | lo;
    }
    for (int b = nblk + lane; b < nwords; b += 32) W[b] = 0;
    ok = __all_sync(kFull, ok);
  } else {
    uint8_t* B = reinterpret_cast<uint8_t*>(W);
    const int nbytes = nwords * 8;
    for (int i = lane; i < nbytes; i += 32) {
      const uint8_t c = i < len ? src[i] : 0;
      B[(i & ~7) | (7 - (i & 7))] = c;  // big-endian inside each word
    }
  }
  __syncwarp();
  return ok;
}

// ------------------------------------------------------------------ kernel
template <typename OffT>
struct WarpMem {
  uint64_t* P;
  uint64_t* T;
  int2* meta;    // [nrows] trimmed (lo,hi) of each ring row; lo>hi == empty
  OffT* ring;    // [nrows][wcap]
  int2* table;   // [table_cap] back-trace row table (choice-byte base, lo)
  uint8_t* bits; // [bits_cap] back-trace choice bytes
};

template <bool A2P>
__device__ __forceinline__ int num_rows(const Penalties& pen) {
  return A2P ? pen.R + 2 * pen.RI1 + 2 * pen.RI2 : pen.R + 2 * pen.RI1;
}

// NULL-fill a row over [a,b] (positions mod wcap).
template <typename OffT>
__device__ __forceinline__ void null_range(OffT* row, int a, int b, int mask, int lane) {
  for (int k = a + lane; k <= b; k += 32) row[k & mask] = null_of<OffT>();
}

template <bool A2P, bool CIGAR, int ENC, typename OffT>
__global__ void __launch_bounds__(256) wfa_align_kernel(const KParams p) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int64_t gwarp = (int64_t)blockIdx.x * wpc + warp;
  const Penalties pen = p.pen;
  const int nrows = num_rows<A2P>(pen);
  const int wcap = p.wcap;
  const int mask = wcap - 1;
  const int nwords = (ENC == 2) ? ((p.max_len + 31) >> 5) + 2 : ((p.max_len + 7) >> 3) + 2;

  // ---- carve per-warp memory
  WarpMem<OffT> m;
  {
    // shared memory of this warp: [P,T if staged here][meta][ring if here]
    uint8_t* ws = smem + (size_t)warp * p.smem_per_warp;
    uint8_t* gs = p.gscratch ? p.gscratch + gwarp * p.gscratch_per_warp : nullptr;
    if (p.seq_in_smem) {
      m.P = reinterpret_cast<uint64_t*>(ws);
      ws += (size_t)2 * nwords * sizeof(uint64_t);
    } else {
      m.P = reinterpret_cast<uint64_t*>(gs + (p.ring_in_smem ? 0 : p.ring_bytes_global));
    }
    m.T = m.P + nwords;
    m.meta = reinterpret_cast<int2*>(ws);
    ws += (size_t)nrows * sizeof(int2);
    if (p.ring_in_smem) {
      m.ring = reinterpret_cast<OffT*>((reinterpret_cast<uintptr_t>(ws) + 15) & ~uintptr_t(15));
    } else {
      m.ring = reinterpret_cast<OffT*>(gs);
      gs += p.ring_bytes_global;
    }
    if (!p.seq_in_smem) gs += p.seq_bytes_global;
    if (CIGAR) {
      m.table = reinterpret_cast<int2*>(gs);
      m.bits = reinterpret_cast<uint8_t*>(m.table + p.table_cap);
    } else {
      m.table = nullptr;
      m.bits = nullptr;
    }
  }
  // ring starts all-NULL, every row empty
  for (int i = lane; i < nrows * wcap; i += 32) m.ring[i] = null_of<OffT>();
  for (int r = lane; r < nrows; r += 32) m.meta[r] = make_int2(1, 0);
  __syncwarp();

  const int n_items = p.num_items_dev ? *p.num_items_dev : p.n_items;
  const int rowI1 = pen.R, rowD1 = pen.R + pen.RI1;
  const int rowI2 = pen.R + 2 * pen.RI1, rowD2 = rowI2 + pen.RI2;

  while (true) {
    int item = 0;
    if (lane == 0) item = atomicAdd(p.queue, 1);
    item = __shfl_sync(kFull, item, 0);
    if (item >= n_items) break;
    const int pair = p.items ? p.items[item] : item;
    const int plen = p.p_len[pair];
    const int tlen = p.t_len[pair];

    // ---- reset ring rows used by the previous pair
    for (int r = 0; r < nrows; ++r) {
      const int2 mt = m.meta[r];
      if (mt.x <= mt.y) null_range(m.ring + (size_t)r * wcap, mt.x, mt.y, mask, lane);
    }
    __syncwarp();
    for (int r = lane; r < nrows; r += 32) m.meta[r] = make_int2(1, 0);

    // ---- stage sequences
    bool ok = true;
    if (plen > p.max_len || tlen > p.max_len) ok = false;
    if (ok) {
      ok &= stage_sequence<ENC>(p.seqs + p.p_off[pair], plen, m.P, nwords, lane);
      ok &= stage_sequence<ENC>(p.seqs + p.t_off[pair], tlen, m.T, nwords, lane);
    }
    if (!ok) {
      if (lane == 0) {
        if (p.final_pass) {
          p.status[pair] = kStOOM;
          p.scores[pair] = 0;
          if (CIGAR) p.ops_len[pair] = 0;
        } else {
          p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
        }
      }
      __syncwarp();
      continue;
    }

    // ---- score 0: M[0][0] = 0 (wavefront/wavefront_aligner.c:236-253)
    OffT* const rowM0 = m.ring;  // slot 0
    if (lane == 0) {
      rowM0[0] = 0;
      m.meta[0] = make_int2(0, 0);
      if (CIGAR) m.table[0] = make_int2(0, 0);
    }
    __syncwarp();

    int s = 0;
    int curM = 0, cur1 = 0, cur2 = 0;  // ring slots of score s
    int null_steps = 0;
    int64_t cursor = 0;  // choice bytes used
    int result = 0;      // 1 done, -1 overflow, 2 max steps, 3 unreachable
    const int k_end = tlen - plen;
    int mlo = 0, mhi = 0;  // trimmed limits of M[s]
    bool m_exists = true;

    while (true) {
      // ================= extend M[s] and test termination
      if (m_exists) {
        OffT* rowM = m.ring + (size_t)curM * wcap;
        for (int k = mlo + lane; k <= mhi; k += 32) {
          const int32_t off = rowM[k & mask];
          if (off >= 0) {
            const int v = off - k;
            const int lim = min(plen - v, tlen - off);
            const int L = lcp<ENC>(m.P, m.T, v, off, lim);
            if (L) rowM[k & mask] = (OffT)(off + L);
          }
        }
        __syncwarp();
        if (mlo <= k_end && k_end <= mhi && (int32_t)rowM[k_end & mask] >= tlen) {
          result = 1;
          break;
        }
      } else if (null_steps > pen.R) {
        result = 3;
        break;
      }

      // ================= compute score s+1
      ++s;
      // no end-to-end alignment scores above the reference's bound
      // (wavefront/wavefront_components.c:101-108): a guard, never hit
      if (s > p.table_cap) {
        result = 4;
        break;
      }
      curM = (curM + 1 == pen.R) ? 0 : curM + 1;
      cur1 = (cur1 + 1 == pen.RI1) ? 0 : cur1 + 1;
      if (A2P) cur2 = (cur2 + 1 == pen.RI2) ? 0 : cur2 + 1;

      // input rows (score < 0 -> empty)
      const int sMx = ring_mod_back(curM, pen.x, pen.R);
      const int sMo1 = ring_mod_back(curM, pen.o1 + pen.e1, pen.R);
      const int sI1 = ring_mod_back(cur1, pen.e1, pen.RI1);
      const int2 eMx = (s - pen.x >= 0) ? m.meta[sMx] : make_int2(1, 0);
      const int2 eMo1 = (s - pen.o1 - pen.e1 >= 0) ? m.meta[sMo1] : make_int2(1, 0);
      const int2 eI1 = (s - pen.e1 >= 0) ? m.meta[rowI1 + sI1] : make_int2(1, 0);
      const int2 eD1 = (s - pen.e1 >= 0) ? m.meta[rowD1 + sI1] : make_int2(1, 0);
      int sMo2 = 0, sI2 = 0;
      int2 eMo2 = make_int2(1, 0), eI2 = make_int2(1, 0), eD2 = make_int2(1, 0);
      if (A2P) {
        sMo2 = ring_mod_back(curM, pen.o2 + pen.e2, pen.R);
        sI2 = ring_mod_back(cur2, pen.e2, pen.RI2);
        if (s - pen.o2 - pen.e2 >= 0) eMo2 = m.meta[sMo2];
        if (s - pen.e2 >= 0) {
          eI2 = m.meta[rowI2 + sI2];
          eD2 = m.meta[rowD2 + sI2];
        }
      }
      const bool vMx = eMx.x <= eMx.y, vMo1 = eMo1.x <= eMo1.y;
      const bool vI1 = eI1.x <= eI1.y, vD1 = eD1.x <= eD1.y;
      const bool vMo2 = A2P && eMo2.x <= eMo2.y;
      const bool vI2 = A2P && eI2.x <= eI2.y, vD2 = A2P && eD2.x <= eD2.y;

      // output rows: clear the content left by the score that used the slot
      OffT* oM = m.ring + (size_t)curM * wcap;
      OffT* oI1 = m.ring + (size_t)(rowI1 + cur1) * wcap;
      OffT* oD1 = m.ring + (size_t)(rowD1 + cur1) * wcap;
      OffT* oI2 = A2P ? m.ring + (size_t)(rowI2 + cur2) * wcap : nullptr;
      OffT* oD2 = A2P ? m.ring + (size_t)(rowD2 + cur2) * wcap : nullptr;

      // wavefront/wavefront_compute_affine.c:236-243: all inputs null -> null step
      if (!(vMx | vMo1 | vI1 | vD1 | vMo2 | vI2 | vD2)) {
        ++null_steps;
        {
          int2 t = m.meta[curM];
          if (t.x <= t.y) null_range(oM, t.x, t.y, mask, lane);
          t = m.meta[rowI1 + cur1];
          if (t.x <= t.y) null_range(oI1, t.x, t.y, mask, lane);
          t = m.meta[rowD1 + cur1];
          if (t.x <= t.y) null_range(oD1, t.x, t.y, mask, lane);
          if (A2P) {
            t = m.meta[rowI2 + cur2];
            if (t.x <= t.y) null_range(oI2, t.x, t.y, mask, lane);
            t = m.meta[rowD2 + cur2];
            if (t.x <= t.y) null_range(oD2, t.x, t.y, mask, lane);
          }
        }
        __syncwarp();
        if (lane == 0) {
          m.meta[curM] = make_int2(1, 0);
          m.meta[rowI1 + cur1] = make_int2(1, 0);
          m.meta[rowD1 + cur1] = make_int2(1, 0);
          if (A2P) {
            m.meta[rowI2 + cur2] = make_int2(1, 0);
            m.meta[rowD2 + cur2] = make_int2(1, 0);
          }
        }
        if (CIGAR) {
          if (s >= p.table_cap) {
            result = -1;
            break;
          }
          if (lane == 0) m.table[s] = make_int2(-1, 0);
        }
        __syncwarp();
        m_exists = false;
        if (s >= p.max_steps) {
          result = 2;
          break;
        }
        continue;
      }
      null_steps = 0;

      // wavefront/wavefront_compute.c:40-87: output range
      int lo = INT32_MAX, hi = INT32_MIN;
      if (vMx) { lo = min(lo, eMx.x); hi = max(hi, eMx.y); }
      if (vMo1) { lo = min(lo, eMo1.x - 1); hi = max(hi, eMo1.y + 1); }
      if (vI1) { lo = min(lo, eI1.x + 1); hi = max(hi, eI1.y + 1); }
      if (vD1) { lo = min(lo, eD1.x - 1); hi = max(hi, eD1.y - 1); }
      if (A2P) {
        if (vMo2) { lo = min(lo, eMo2.x - 1); hi = max(hi, eMo2.y + 1); }
        if (vI2) { lo = min(lo, eI2.x + 1); hi = max(hi, eI2.y + 1); }
        if (vD2) { lo = min(lo, eD2.x - 1); hi = max(hi, eD2.y - 1); }
      }
      const int width = hi - lo + 1;
      if (width + 2 > wcap) {
        result = -1;
        break;
      }
      if (CIGAR) {
        if (s >= p.table_cap || cursor + width > p.bits_cap) {
          result = -1;
          break;
        }
      }
      // clear old content of the output slots outside [lo,hi]
      {
        int2 t = m.meta[curM];
        if (t.x <= t.y) {
          null_range(oM, t.x, min(t.y, lo - 1), mask, lane);
          null_range(oM, max(t.x, hi + 1), t.y, mask, lane);
        }
        t = m.meta[rowI1 + cur1];
        if (t.x <= t.y) {
          null_range(oI1, t.x, min(t.y, lo - 1), mask, lane);
          null_range(oI1, max(t.x, hi + 1), t.y, mask, lane);
        }
        t = m.meta[rowD1 + cur1];
        if (t.x <= t.y) {
          null_range(oD1, t.x, min(t.y, lo - 1), mask, lane);
          null_range(oD1, max(t.x, hi + 1), t.y, mask, lane);
        }
        if (A2P) {
          t = m.meta[rowI2 + cur2];
          if (t.x <= t.y) {
            null_range(oI2, t.x, min(t.y, lo - 1), mask, lane);
            null_range(oI2, max(t.x, hi + 1), t.y, mask, lane);
          }
          t = m.meta[rowD2 + cur2];
          if (t.x <= t.y) {
            null_range(oD2, t.x, min(t.y, lo - 1), mask, lane);
            null_range(oD2, max(t.x, hi + 1), t.y, mask, lane);
          }
        }
      }
      __syncwarp();

      // input row pointers; a null input reads as all-NULL: point it at an
      // output row position range that is NULL?  Simpler: select per read.
      const OffT* rMx = m.ring + (size_t)sMx * wcap;
      const OffT* rMo1 = m.ring + (size_t)sMo1 * wcap;
      const OffT* rI1 = m.ring + (size_t)(rowI1 + sI1) * wcap;
      const OffT* rD1 = m.ring + (size_t)(rowD1 + sI1) * wcap;
      const OffT* rMo2 = A2P ? m.ring + (size_t)sMo2 * wcap : nullptr;
      const OffT* rI2 = A2P ? m.ring + (size_t)(rowI2 + sI2) * wcap : nullptr;
      const OffT* rD2 = A2P ? m.ring + (size_t)(rowD2 + sI2) * wcap : nullptr;
      uint8_t* brow = CIGAR ? m.bits + cursor - lo : nullptr;

      int tloM = INT32_MAX, thiM = INT32_MIN;
      int tloI1 = INT32_MAX, thiI1 = INT32_MIN, tloD1 = INT32_MAX, thiD1 = INT32_MIN;
      int tloI2 = INT32_MAX, thiI2 = INT32_MIN, tloD2 = INT32_MAX, thiD2 = INT32_MIN;
      for (int k = lo + lane; k <= hi; k += 32) {
        const int km = (k - 1) & mask, k0 = k & mask, kp = (k + 1) & mask;
        // empty input rows read as NULL (a stale slot is never read)
        const int32_t mo1_m = vMo1 ? rMo1[km] : kNull;
        const int32_t mo1_p = vMo1 ? rMo1[kp] : kNull;
        const int32_t i1_e = vI1 ? rI1[km] : kNull;
        const int32_t d1_e = vD1 ? rD1[kp] : kNull;
        const int32_t mx = vMx ? rMx[k0] : kNull;
        // wavefront/wavefront_compute_affine.c:66-84
        int32_t i1 = max(mo1_m, i1_e) + 1;
        int32_t d1 = max(mo1_p, d1_e);
        const int32_t mis = mx + 1;
        int32_t ins = i1, del = d1;
        int32_t i2 = kNull, d2 = kNull;
        int32_t mo2_m = kNull, mo2_p = kNull, i2_e = kNull, d2_e = kNull;
        if (A2P) {
          // wavefront/wavefront_compute_affine2p.c:78-95
          mo2_m = vMo2 ? rMo2[km] : kNull;
          mo2_p = vMo2 ? rMo2[kp] : kNull;
          i2_e = vI2 ? rI2[km] : kNull;
          d2_e = vD2 ? rD2[kp] : kNull;
          i2 = max(mo2_m, i2_e) + 1;
          d2 = max(mo2_p, d2_e);
          ins = max(i1, i2);
          del = max(d1, d2);
        }
        int32_t mval = max(del, max(mis, ins));
        if ((uint32_t)mval > (uint32_t)tlen || (uint32_t)(mval - k) > (uint32_t)plen) mval = kNull;
        // canonical NULL for the gap components
        if (i1 < 0) i1 = kNull;
        if (d1 < 0) d1 = kNull;
        put(oM, k0, mval);
        put(oI1, k0, i1);
        put(oD1, k0, d1);
        if (mval >= 0) { tloM = min(tloM, k); thiM = max(thiM, k); }
        if ((uint32_t)i1 <= (uint32_t)tlen && (uint32_t)(i1 - k) <= (uint32_t)plen) {
          tloI1 = min(tloI1, k); thiI1 = max(thiI1, k);
        }
        if ((uint32_t)d1 <= (uint32_t)tlen && (uint32_t)(d1 - k) <= (uint32_t)plen) {
          tloD1 = min(tloD1, k); thiD1 = max(thiD1, k);
        }
        if (A2P) {
          if (i2 < 0) i2 = kNull;
          if (d2 < 0) d2 = kNull;
          put(oI2, k0, i2);
          put(oD2, k0, d2);
          if ((uint32_t)i2 <= (uint32_t)tlen && (uint32_t)(i2 - k) <= (uint32_t)plen) {
            tloI2 = min(tloI2, k); thiI2 = max(thiI2, k);
          }
          if ((uint32_t)d2 <= (uint32_t)tlen && (uint32_t)(d2 - k) <= (uint32_t)plen) {
            tloD2 = min(tloD2, k); thiD2 = max(thiD2, k);
          }
        }
        if (CIGAR) {
          // M source; exact ties: mismatch > D2 > D1 > I2 > I1
          // (wavefront/wavefront_backtrace.c:49-59 type codes)
          const int32_t best = max(mis, max(ins, del));
          uint8_t src;
          if (mis == best) src = kSrcX;
          else if (A2P && d2 == best) src = kSrcD2;
          else if (d1 == best) src = kSrcD1;
          else if (A2P && i2 == best) src = kSrcI2;
          else src = kSrcI1;
          uint8_t c = src;
          c |= (uint8_t)(i1_e >= mo1_m) << 3;
          c |= (uint8_t)(d1_e >= mo1_p) << 4;
          if (A2P) {
            c |= (uint8_t)(i2_e >= mo2_m) << 5;
            c |= (uint8_t)(d2_e >= mo2_p) << 6;
          }
          brow[k] = c;
        }
      }
      __syncwarp();
      tloM = __reduce_min_sync(kFull, tloM);
      thiM = __reduce_max_sync(kFull, thiM);
      tloI1 = __reduce_min_sync(kFull, tloI1);
      thiI1 = __reduce_max_sync(kFull, thiI1);
      tloD1 = __reduce_min_sync(kFull, tloD1);
      thiD1 = __reduce_max_sync(kFull, thiD1);
      if (A2P) {
        tloI2 = __reduce_min_sync(kFull, tloI2);
        thiI2 = __reduce_max_sync(kFull, thiI2);
        tloD2 = __reduce_min_sync(kFull, tloD2);
        thiD2 = __reduce_max_sync(kFull, thiD2);
      }
      // NULL the trimmed-away ends (wavefront/wavefront_compute.c:579-613)
      auto trim_fill = [&](OffT* row, int tlo_, int thi_) {
        if (tlo_ > thi_) {
          null_range(row, lo, hi, mask, lane);
        } else {
          null_range(row, lo, tlo_ - 1, mask, lane);
          null_range(row, thi_ + 1, hi, mask, lane);
        }
      };
      trim_fill(oM, tloM, thiM);
      trim_fill(oI1, tloI1, thiI1);
      trim_fill(oD1, tloD1, thiD1);
      if (A2P) {
        trim_fill(oI2, tloI2, thiI2);
        trim_fill(oD2, tloD2, thiD2);
      }
      __syncwarp();
      if (lane == 0) {
        m.meta[curM] = make_int2(tloM, thiM);
        m.meta[rowI1 + cur1] = make_int2(tloI1, thiI1);
        m.meta[rowD1 + cur1] = make_int2(tloD1, thiD1);
        if (A2P) {
          m.meta[rowI2 + cur2] = make_int2(tloI2, thiI2);
          m.meta[rowD2 + cur2] = make_int2(tloD2, thiD2);
        }
        if (CIGAR) m.table[s] = make_int2((int)cursor, lo);
      }
      if (CIGAR) cursor += width;
      mlo = tloM;
      mhi = thiM;
      m_exists = true;
      __syncwarp();
      // wavefront/wavefront_unialign.c:102-107
      if (s >= p.max_steps) {
        result = 2;
        break;
      }
    }

    // ================= finish the pair
    if (result == -1) {
      if (lane == 0) {
        if (p.final_pass) {
          p.status[pair] = kStOOM;
          p.scores[pair] = 0;
          if (CIGAR) p.ops_len[pair] = 0;
        } else {
          p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
        }
      }
      __syncwarp();
      continue;
    }
    if (result == 2) {
      if (lane == 0) {
        p.status[pair] = kStMaxSteps;
        p.scores[pair] = -p.max_steps;
        if (CIGAR) p.ops_len[pair] = 0;
      }
      __syncwarp();
      continue;
    }
    if (result == 4) {
      if (lane == 0) {
        p.status[pair] = kStUnattainable;
        p.scores[pair] = 0;
        if (CIGAR) p.ops_len[pair] = 0;
      }
      __syncwarp();
      continue;
    }
    if (result == 3) {
      if (lane == 0) {
        p.status[pair] = kStPartial;
        p.scores[pair] = -s;
        if (CIGAR) p.ops_len[pair] = 0;
      }
      __syncwarp();
      continue;
    }
    // classic score (wavefront/wavefront_compute.c:108-120)
    int score;
    if (pen.match == 0) score = -s;
    else score = ((-pen.match) * (plen + tlen) - s) / 2;

    if (!CIGAR) {
      if (lane == 0) {
        p.scores[pair] = score;
        p.status[pair] = kStCompleted;
      }
      __syncwarp();
      continue;
    }

    // ================= back-trace (choice bytes) then forward replay
    if (lane == 0) {
      uint8_t* items = m.bits + cursor;
      const int64_t items_cap = p.bits_cap - cursor;
      int64_t n = 0;
      int st = 0;  // 0 M, 1 I1, 2 D1, 3 I2, 4 D2
      int ss = s, kk = k_end;
      bool bad = false;
      while (true) {
        if (n + 2 > items_cap || ss < 0) { bad = true; break; }
        if (st == 0) {
          items[n++] = 'E';
          if (ss == 0) {
            if (kk != 0) bad = true;
            break;
          }
        }
        const int2 te = m.table[ss];
        const int64_t bi = (int64_t)te.x + (kk - te.y);
        if (te.x < 0 || kk < te.y || bi >= cursor) { bad = true; break; }
        const uint8_t c = m.bits[bi];
        if (st == 0) {
          const int src = c & 7;
          if (src == kSrcX) { items[n++] = 'X'; ss -= pen.x; }
          else if (src == kSrcD1) st = 2;
          else if (src == kSrcI1) st = 1;
          else if (src == kSrcD2) st = 4;
          else st = 3;
        } else if (st == 1) {
          items[n++] = 'I';
          kk -= 1;
          if (c & 8) ss -= pen.e1; else { ss -= pen.o1 + pen.e1; st = 0; }
        } else if (st == 2) {
          items[n++] = 'D';
          kk += 1;
          if (c & 16) ss -= pen.e1; else { ss -= pen.o1 + pen.e1; st = 0; }
        } else if (st == 3) {
          items[n++] = 'I';
          kk -= 1;
          if (c & 32) ss -= pen.e2; else { ss -= pen.o2 + pen.e2; st = 0; }
        } else {
          items[n++] = 'D';
          kk += 1;
          if (c & 64) ss -= pen.e2; else { ss -= pen.o2 + pen.e2; st = 0; }
        }
      }
      int out_n = 0;
      if (!bad) {
        uint8_t* out = p.ops + p.ops_off[pair];
        int v = 0, h = 0;
        for (int64_t i = n - 1; i >= 0; --i) {
          const uint8_t it = items[i];
          if (it == 'E') {
            const int L = lcp<ENC>(m.P, m.T, v, h, min(plen - v, tlen - h));
            for (int j = 0; j < L; ++j) out[out_n++] = 'M';
            v += L;
            h += L;
          } else if (it == 'X') {
            if (v >= plen || h >= tlen) { bad = true; break; }
            out[out_n++] = 'X'; ++v; ++h;
          } else if (it == 'I') {
            if (h >= tlen) { bad = true; break; }
            out[out_n++] = 'I'; ++h;
          } else {
            if (v >= plen) { bad = true; break; }
            out[out_n++] = 'D'; ++v;
          }
        }
        if (v != plen || h != tlen) bad = true;
      }
      if (bad) {
        p.status[pair] = kStUnattainable;
        p.scores[pair] = score;
        p.ops_len[pair] = 0;
      } else {
        p.status[pair] = kStCompleted;
        p.scores[pair] = score;
        p.ops_len[pair] = out_n;
      }
    }
    __syncwarp();
  }
}

// -------------------------------------------------------------- launchers
#define WF2G_INST(A2P, CIG, ENC, T) template __global__ void wfa_align_kernel<A2P, CIG, ENC, T>(const KParams p);
#define WF2G_INST_T(T)               \
  WF2G_INST(false, false, 2, T)      \
  WF2G_INST(false, true, 2, T)       \
  WF2G_INST(true, false, 2, T)       \
  WF2G_INST(true, true, 2, T)        \
  WF2G_INST(false, false, 8, T)      \
  WF2G_INST(false, true, 8, T)       \
  WF2G_INST(true, false, 8, T)       \
  WF2G_INST(true, true, 8, T)
WF2G_INST_T(int16_t)
WF2G_INST_T(int32_t)

template <typename T>
static void* pick(int a2p, int cigar, int enc) {
  if (enc == 2) {
    if (!a2p) return cigar ? (void*)wfa_align_kernel<false, true, 2, T> : (void*)wfa_align_kernel<false, false, 2, T>;
    return cigar ? (void*)wfa_align_kernel<true, true, 2, T> : (void*)wfa_align_kernel<true, false, 2, T>;
  }
  if (!a2p) return cigar ? (void*)wfa_align_kernel<false, true, 8, T> : (void*)wfa_align_kernel<false, false, 8, T>;
  return cigar ? (void*)wfa_align_kernel<true, true, 8, T> : (void*)wfa_align_kernel<true, false, 8, T>;
}

// Kernel variant for (affine2p?, full CIGAR?, 2- or 8-bit sequences, 2- or 4-byte offsets).
extern "C" void* wf2g_kernel_ptr(int a2p, int cigar, int enc, int off_bytes) {
  return off_bytes == 2 ? pick<int16_t>(a2p, cigar, enc) : pick<int32_t>(a2p, cigar, enc);
}

}  // namespace wf2g

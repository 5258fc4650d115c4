// wfa_align.cuh -- the alignment kernel of the GB300 wavefront aligner and
// its device helpers, as a template included by the units that instantiate
// it (wfa_kernels.cu: a warp per pair, exact; wfa_kernels_heur.cu: a warp per
// pair, wf-adaptive; wfa_kernels_wide.cu: a CTA per pair).
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
// GPU design: a group of G threads per pair (a warp, or a 256-thread CTA for
// long pairs), threads striped over diagonals k.  Every wavefront row is NULL
// outside its trimmed range (the reference's NULL padding,
// wavefront/wavefront_compute.c:498-575), so the cell loop reads its inputs
// without bounds checks; empty inputs read an all-NULL row.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "wfa_kernels.cuh"

namespace wf2g {


// NULL as stored in a row of OffT (int16 rows serve sequences < 32000).
template <typename OffT>
__device__ __forceinline__ OffT null_of() {
  return sizeof(OffT) == 2 ? (OffT)(-32768) : (OffT)kNull;
}

// ---------------------------------------------------------------- checking
// Built with -DWF2G_CHECKED every ring, sequence, back-trace and output access
// is bounds-checked: a violation is recorded (first one wins) and the access
// is skipped, so a faulty index is reported instead of faulting the GPU.
#ifdef WF2G_CHECKED
static __device__ unsigned long long g_fault[4];  // site, index, pair, count (per unit)
__device__ __forceinline__ bool wf2g_ok(bool ok, int site, long long idx, int pair) {
  if (!ok) {
    if (atomicCAS(&g_fault[0], 0ull, (unsigned long long)site) == 0ull) {
      g_fault[1] = (unsigned long long)idx;
      g_fault[2] = (unsigned long long)pair;
    }
    atomicAdd(&g_fault[3], 1ull);
  }
  return ok;
}
#define CHK(cond, site, idx) wf2g_ok((cond), (site), (long long)(idx), g_pair)
#else
#define CHK(cond, site, idx) true
#endif

// Each unit that instantiates the kernel exports a reader of its own record.
#ifdef WF2G_CHECKED
#define WF2G_FAULT_READER(name)                                                   \
  extern "C" int name(unsigned long long* out) {                                 \
    return (int)cudaMemcpyFromSymbol(out, g_fault, 4 * sizeof(unsigned long long)); \
  }
#else
#define WF2G_FAULT_READER(name)                  \
  extern "C" int name(unsigned long long* out) { \
    for (int i = 0; i < 4; ++i) out[i] = 0;      \
    return 0;                                    \
  }
#endif

// a - b in wrapping int32 arithmetic: the reference computes score
// differences in int, where an INT_MIN best overflows
__device__ __forceinline__ int wsub32(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }

__device__ __forceinline__ int ring_back(int cur, int d, int R) {
  // slot of score (s-d) when the slot of s is cur, 0 <= d < R
  const int t = cur - d;
  return t < 0 ? t + R : t;
}

// ---------------------------------------------------------------- sequences
// ENC==2: base i at bits [31-2(i%16), 30-2(i%16)] of 32-bit word i/16.
// ENC==8: byte i at bits [63-8(i%8), 56-8(i%8)] of 64-bit word i/8.
template <int ENC>
struct Seq;

template <>
struct Seq<2> {
  typedef uint32_t Word;
  static constexpr int kPer = 16;
  static __device__ __forceinline__ uint32_t window(const uint32_t* W, int pos) {
    const int w = pos >> 4;
    return __funnelshift_l(W[w + 1], W[w], (pos & 15) << 1);
  }
  static __device__ __forceinline__ int equal_prefix(uint32_t d) { return __clz(d) >> 1; }
  static __host__ __device__ int words(int len) { return ((len + 15) >> 4) + 2; }
};

template <>
struct Seq<8> {
  typedef uint64_t Word;
  static constexpr int kPer = 8;
  static __device__ __forceinline__ uint64_t window(const uint64_t* W, int pos) {
    const int w = pos >> 3;
    const int sh = (pos & 7) << 3;
    uint64_t x = W[w];
    if (sh) x = (x << sh) | (W[w + 1] >> (64 - sh));
    return x;
  }
  static __device__ __forceinline__ int equal_prefix(uint64_t d) { return __clzll(d) >> 3; }
  static __host__ __device__ int words(int len) { return ((len + 7) >> 3) + 2; }
};

// Longest common prefix of P[v..] and T[h..], at most lim characters:
// word-wide XOR + count-leading-zeros (wavefront/wavefront_extend_kernels.c:68-92).
template <int ENC>
__device__ __forceinline__ int lcp(const typename Seq<ENC>::Word* P,
                                   const typename Seq<ENC>::Word* T, int v, int h, int lim,
                                   int nw = 0, int g_pair = 0) {
  int L = 0;
  while (L < lim) {
    const int wp = (v + L) / Seq<ENC>::kPer, wt = (h + L) / Seq<ENC>::kPer;
    if (!CHK(v + L >= 0 && wp + 1 < nw, 20, v + L) || !CHK(h + L >= 0 && wt + 1 < nw, 21, h + L))
      return 0;
    const auto d = Seq<ENC>::window(P, v + L) ^ Seq<ENC>::window(T, h + L);
    if (d) {
      L += Seq<ENC>::equal_prefix(d);
      break;
    }
    L += Seq<ENC>::kPer;
  }
  return L < lim ? L : lim;
}

// Group barrier: a warp (G == 32) or the whole CTA (one group per CTA).
template <int G>
__device__ __forceinline__ void group_sync() {
  if (G == 32) __syncwarp();
  else __syncthreads();
}

// Stages one sequence into W (group-cooperative; t is the thread's rank in
// its group of G threads).  Returns false if ENC==2 and the sequence holds a
// byte outside {A,C,G,T}.
template <int ENC, int G>
__device__ bool stage_sequence(const uint8_t* __restrict__ src, int len,
                               typename Seq<ENC>::Word* W, int t) {
  const int nwords = Seq<ENC>::words(len);
  const int lane = t & 31;
  bool ok = true;
  if (ENC == 2) {
    const int nblk = (len + 31) >> 5;  // 32 bases -> 2 words, one warp each
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
      if (lane == 0) {
        W[2 * b] = w0;
        if (2 * b + 1 < nwords) W[2 * b + 1] = w1;
      }
    }
    for (int b = 2 * nblk + t; b < nwords; b += G) W[b] = 0;
    if (G == 32) ok = __all_sync(kFull, ok);
    else ok = __syncthreads_and(ok);
  } else {
    uint8_t* B = reinterpret_cast<uint8_t*>(W);
    const int nbytes = nwords * 8;
    for (int i = t; i < nbytes; i += G) {
      const uint8_t c = i < len ? src[i] : 0;
      B[(i & ~7) | (7 - (i & 7))] = c;  // big-endian inside each word
    }
  }
  group_sync<G>();
  return ok;
}

// Ring bounds of the calling group (checked builds only).
struct RingBounds {
  const void* lo;
  const void* hi;
};

// NULL-fill row elements of diagonals [a,b] (group-cooperative).
template <typename OffT, int G>
__device__ __forceinline__ void null_range(OffT* row, int a, int b, int t,
                                           RingBounds rb = RingBounds{nullptr, nullptr},
                                           int g_pair = 0) {
  if (a > b) return;  // also keeps a + t from overflowing on empty ranges
  for (int k = a + t; k <= b; k += G) {
    if (CHK(rb.lo == nullptr || ((const void*)(row + k) >= rb.lo && (const void*)(row + k) < rb.hi), 1, k))
      row[k] = null_of<OffT>();
  }
}

// After computing [lo,hi] and finding the trimmed range [tlo,thi]: NULL the
// trimmed-away ends (wavefront/wavefront_compute.c:579-613).
template <typename OffT, int G>
__device__ __forceinline__ void trim_fill(OffT* row, int lo, int hi, int tlo, int thi, int t,
                                          RingBounds rb, int g_pair) {
  if (tlo == lo && thi == hi) return;  // nothing trimmed (the usual case)
  if (tlo > thi) {
    null_range<OffT, G>(row, lo, hi, t, rb, g_pair);
  } else {
    null_range<OffT, G>(row, lo, tlo - 1, t, rb, g_pair);
    null_range<OffT, G>(row, thi + 1, hi, t, rb, g_pair);
  }
}

// Clears what a reused slot holds outside the new range [lo,hi].
template <typename OffT, int G>
__device__ __forceinline__ void clear_outside(OffT* row, int2 old, int lo, int hi, int t,
                                              RingBounds rb, int g_pair) {
  // nothing outside [lo,hi] to clear when the old window lies inside it (the
  // usual case: wavefronts grow) or is empty
  if (old.x <= old.y && (old.x < lo || old.y > hi)) {
    null_range<OffT, G>(row, old.x, min(old.y, lo - 1), t, rb, g_pair);
    null_range<OffT, G>(row, max(old.x, hi + 1), old.y, t, rb, g_pair);
  }
}

__device__ __forceinline__ bool in_bounds(int32_t off, int k, int plen, int tlen) {
  return (uint32_t)off <= (uint32_t)tlen && (uint32_t)(off - k) <= (uint32_t)plen;
}

// ---------------------------------------------------------------- block pool
// A spin lock with a bounded number of tries guards the free stack; a caller
// that gives up treats the pool as empty (its pair is retried in a later pass).
constexpr int kPoolTries = 1 << 20;

__device__ __forceinline__ bool pool_lock(int32_t* lock) {
  for (int i = 0; i < kPoolTries; ++i) {
    if (atomicCAS(lock, 0, 1) == 0) {
      __threadfence();
      return true;
    }
    __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void pool_unlock(int32_t* lock) {
  __threadfence();
  atomicExch(lock, 0);
}
// One free block index, or -1.
__device__ __forceinline__ int pool_pop(const KParams& p) {
  if (!pool_lock(p.pool_lock)) return -1;
  volatile int32_t* const cnt = p.pool_count;
  volatile int32_t* const stk = p.pool_stack;
  int b = -1;
  const int c = *cnt;
  if (c > 0) {
    b = stk[c - 1];
    *cnt = c - 1;
  }
  pool_unlock(p.pool_lock);
  return b;
}
// Returns n blocks (if the lock cannot be had they stay out of the pool until
// the next batch re-initialises it).
__device__ __forceinline__ void pool_push(const KParams& p, const int32_t* blocks, int n) {
  if (!pool_lock(p.pool_lock)) return;
  volatile int32_t* const cnt = p.pool_count;
  volatile int32_t* const stk = p.pool_stack;
  const int c = *cnt;
  for (int i = 0; i < n; ++i) stk[c + i] = blocks[i];
  *cnt = c + n;
  pool_unlock(p.pool_lock);
}


// ---------------------------------------------------------------- extension
// Score of an operation run under the user's penalties as maximal-score
// trimming counts it: a match earns -match, or 1 when match is 0
// (alignment/cigar_utils.c:208-235).
__device__ __forceinline__ int run_score_2p(const KParams& p, uint8_t op, int len, int* ev, int* eh) {
  if (op == 'M') { *ev += len; *eh += len; return (p.um != 0 ? p.um : -1) * len; }
  if (op == 'X') { *ev += len; *eh += len; return p.ux * len; }
  if (op == 'D') *ev += len; else *eh += len;
  return min(p.uo1 + p.ue1 * len, p.uo2 + p.ue2 * len);
}

// Maximal-score trimming of ops[0..*n) (alignment/cigar_utils.c:112-318):
// keeps the highest-scoring prefix; *n, *score, *ev, *eh describe it (an empty
// prefix: 0 ops, INT32_MIN, end (-1,-1), as cigar_clear leaves them).
// Returns whether the CIGAR was trimmed.  Affine2p leaves an empty CIGAR
// untouched and returns false.  One thread, sequential.
template <bool A2P>
__device__ bool maxtrim(const KParams& p, const uint8_t* ops, int* n, int* score, int* ev, int* eh) {
  const int len = *n;
  int max_score = 0, max_off = 0, max_v = 0, max_h = 0, sc = 0, v = 0, h = 0;
  if (A2P) {
    if (len <= 0) return false;
    uint8_t last = 0;
    int run = 0;
    for (int i = 0; i < len; ++i) {
      const uint8_t op = ops[i];
      if (op != last && last != 0) {
        sc -= run_score_2p(p, last, run, &v, &h);
        run = 0;
        if (max_score < sc) { max_score = sc; max_off = i - 1; max_v = v; max_h = h; }
      }
      last = op;
      ++run;
    }
    sc -= run_score_2p(p, last, run, &v, &h);
    if (max_score < sc) { max_score = sc; max_off = len - 1; max_v = v; max_h = h; }
  } else {
    const int msc = p.um != 0 ? p.um : -1;
    uint8_t last = 0;
    for (int i = 0; i < len; ++i) {
      const uint8_t op = ops[i];
      if (op == 'M') { sc -= msc; ++v; ++h; }
      else if (op == 'X') { sc -= p.ux; ++v; ++h; }
      else if (op == 'I') { sc -= p.ue1 + (last == 'I' ? 0 : p.uo1); ++h; }
      else { sc -= p.ue1 + (last == 'D' ? 0 : p.uo1); ++v; }
      last = op;
      if (max_score < sc) { max_score = sc; max_off = i; max_v = v; max_h = h; }
    }
  }
  const bool trimmed = (max_off != len - 1);
  if (max_score == 0) {
    *n = 0;
    *score = INT32_MIN;
    *ev = -1;
    *eh = -1;
  } else {
    *n = max_off + 1;
    *score = max_score;
    *ev = max_v;
    *eh = max_h;
  }
  return trimmed;
}

// Maximal-score trimming under gap-linear penalties (alignment/cigar_utils.c:
// 112-160): um, ux and the indel penalty uo1; same conventions as maxtrim.
// Edit and indel are not trimmed; for them this returns false untouched.
__device__ __forceinline__ bool maxtrim_linear(const KParams& p, const uint8_t* ops, int* n,
                                               int* score, int* ev, int* eh) {
  if (p.metric != 2) return false;
  const int len = *n, msc = p.um != 0 ? p.um : -1;
  int max_score = 0, max_off = 0, max_v = 0, max_h = 0, sc = 0, v = 0, h = 0;
  for (int i = 0; i < len; ++i) {
    const uint8_t op = ops[i];
    if (op == 'M') { sc -= msc; ++v; ++h; }
    else if (op == 'X') { sc -= p.ux; ++v; ++h; }
    else if (op == 'I') { sc -= p.uo1; ++h; }
    else { sc -= p.uo1; ++v; }
    if (max_score < sc) { max_score = sc; max_off = i; max_v = v; max_h = h; }
  }
  const bool trimmed = (max_off != len - 1);
  if (max_score == 0) {
    *n = 0;
    *score = INT32_MIN;
    *ev = -1;
    *eh = -1;
  } else {
    *n = max_off + 1;
    *score = max_score;
    *ev = max_v;
    *eh = max_h;
  }
  return trimmed;
}

// 4 resident 256-thread blocks per SM (64 registers per thread): the kernel
// is latency-bound, so residency matters more than registers.
#ifndef WF2G_MIN_BLOCKS
#define WF2G_MIN_BLOCKS 4
#endif

// HEUR: the wf-adaptive heuristic is compiled in (exact runs do without it).
// G: threads per pair -- 32 (a warp per pair, several groups per CTA) or 256
// (the whole CTA per pair, for long pairs whose rows span thousands of
// diagonals).  For G > 32 the back-trace walk and replay run on the group's
// first warp while the others wait.
// EF: the ends-free form (and its extension variant) is compiled in.
// LIN: the single-component metrics (indel, edit, gap-linear; with A2P false).
template <bool A2P, bool CIGAR, int ENC, typename OffT, bool HEUR, int G, bool EF = false,
          bool LIN = false>
__global__ void __launch_bounds__(256, WF2G_MIN_BLOCKS) wfa_align_kernel(const KParams p) {
  static_assert(G == 32 || G == 256, "a pair is aligned by a warp or a 256-thread CTA");
  typedef typename Seq<ENC>::Word Word;
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31;
  const int t = threadIdx.x % G;      // rank in the group
  const int wig = t >> 5;             // warp in the group
  const int gpc = blockDim.x / G;     // groups per CTA
  const int64_t grp = (int64_t)blockIdx.x * gpc + threadIdx.x / G;
  const Penalties pen = p.pen;
  const int nrows = A2P ? pen.R + 2 * pen.RI1 + 2 * pen.RI2 : pen.R + 2 * pen.RI1;
  const int stride = p.row_stride;
  const int kofs = p.kofs;
  const int nwords = Seq<ENC>::words(p.max_len);

  // ---- carve per-group memory
  uint8_t* ws = smem + (size_t)(threadIdx.x / G) * p.smem_per_group;
  uint8_t* gs = p.gscratch + grp * p.gscratch_per_group;
  OffT* const ring = reinterpret_cast<OffT*>(gs);  // (nrows+1) rows; row nrows is all-NULL
  gs += p.ring_bytes;
  Word* P;
  if (p.seq_in_smem) {
    P = reinterpret_cast<Word*>(ws);
    ws += (size_t)2 * nwords * sizeof(Word);
  } else {
    P = reinterpret_cast<Word*>(gs);
    gs += p.seq_bytes;
  }
  Word* const T = P + nwords;
  int2* const meta = reinterpret_cast<int2*>(ws);  // [nrows] limits (lo,hi); lo>hi == null
  // [nrows] initialised windows: a row is NULL outside its window.  The window
  // equals the limits except after a heuristic cut-off, which narrows only the
  // limits; the cut offsets stay readable, as wf_elements_init_min/max keep
  // them in the reference (wavefront/wavefront_compute.c:498-527)
  int2* const imeta = meta + nrows;
  // G > 32: per-warp partial reductions [G/32][kRedVals] and a broadcast slot
  int32_t* const gred = reinterpret_cast<int32_t*>(imeta + nrows);
  constexpr int kRedVals = 12, kBc = (G / 32) * kRedVals;  // [10] ends-free k, [11] edit pruning
  // single-component metrics (indel, edit, gap-linear): only M rows carry
  // wavefronts; indel has no mismatch; edit and indel follow the edit driver
  // (wavefront/wavefront_compute_edit.c:321-374)
  static_assert(!(LIN && A2P), "the single-component metrics have no second gap model");
  constexpr bool lin = LIN;
  const bool edit_like = LIN && p.metric <= 1;
  const bool has_x = !LIN || p.metric != 0;
  // end-to-end edit prunes wide wavefronts (wavefront/wavefront_compute_edit.c:362-366)
  const bool prune = LIN && !EF && p.metric == 1;
  (void)gred;
  BtRow* const table = CIGAR ? reinterpret_cast<BtRow*>(gs) : nullptr;
  uint8_t* const bits = CIGAR ? reinterpret_cast<uint8_t*>(table + p.table_cap) : nullptr;
  // where choice bytes live: the group's slice, or the shared block pool, in
  // which case the slice holds the pair's block list and then the walk items
  const bool pooled = CIGAR && G > 32 && p.pool != nullptr;  // pooled passes run a CTA per pair
  uint8_t* const bt = pooled ? p.pool : bits;
  int32_t* const owned = reinterpret_cast<int32_t*>(bits);
  const int64_t owned_bytes = pooled ? (int64_t)p.max_blocks * 4 : 0;
  auto row = [=](int r) -> OffT* { return ring + (size_t)r * stride + kofs; };
  const OffT* const null_row = row(nrows);
  const RingBounds rb{ring, ring + (size_t)(nrows + 1) * stride};
  int g_pair = -1;
  (void)rb;
  (void)g_pair;
#ifdef WF2G_CHECKED
#define RING_OK(ptr) CHK((const void*)(ptr) >= rb.lo && (const void*)(ptr) < rb.hi, 2, (const OffT*)(ptr) - ring)
#define RING_LD(r, k) (RING_OK((r) + (k)) ? (int32_t)(r)[k] : (int32_t)null_of<OffT>())
#define RING_ST(r, k, v) do { if (RING_OK((r) + (k))) (r)[k] = (v); } while (0)
#else
#define RING_LD(r, k) ((int32_t)(r)[k])
#define RING_ST(r, k, v) ((r)[k] = (v))
#endif

  // group-wide min / max / broadcast from rank 0 (barriers only for G > 32)
  auto gmin = [&](int x) -> int {
    x = __reduce_min_sync(kFull, x);
    if (G > 32) {
      if (lane == 0) gred[wig] = x;
      __syncthreads();
      x = gred[0];
      for (int w = 1; w < G / 32; ++w) x = min(x, gred[w]);
      __syncthreads();
    }
    return x;
  };
  auto gmax = [&](int x) -> int {
    x = __reduce_max_sync(kFull, x);
    if (G > 32) {
      if (lane == 0) gred[wig] = x;
      __syncthreads();
      x = gred[0];
      for (int w = 1; w < G / 32; ++w) x = max(x, gred[w]);
      __syncthreads();
    }
    return x;
  };
  auto gbcast = [&](int x) -> int {
    if (G == 32) return __shfl_sync(kFull, x, 0);
    if (t == 0) gred[kBc] = x;
    __syncthreads();
    x = gred[kBc];
    __syncthreads();
    return x;
  };

  // ring starts all-NULL, every row empty
  for (int64_t i = t; i < (int64_t)(nrows + 1) * stride; i += G) ring[i] = null_of<OffT>();
  for (int r = t; r < nrows; r += G) meta[r] = imeta[r] = make_int2(1, 0);
  group_sync<G>();

  const int n_items = p.num_items_dev ? *p.num_items_dev : p.n_items;

  while (true) {
    int item = 0;
    if (t == 0) item = atomicAdd(p.queue, 1);
    item = gbcast(item);
    if (item >= n_items) break;
    const int pair = p.items ? p.items[item] : item;
    g_pair = pair;
    const int plen = p.p_len[pair];
    const int tlen = p.t_len[pair];
    if (p.wide_min_len > 0 && max(plen, tlen) >= p.wide_min_len) {
      if (t == 0) p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
      group_sync<G>();
      continue;
    }
    // ends-free lengths of this pair: the extension presets
    // (wavefront/wavefront_align.c:57-63), checked as :90-101 checks them
    int pbf = 0, pef = 0, tbf = 0, tef = 0;
    if (EF) {
      pbf = p.extension ? 0 : p.pbf;
      pef = p.extension ? plen : p.pef;
      tbf = p.extension ? 0 : p.tbf;
      tef = p.extension ? tlen : p.tef;
      if (pbf > plen || pef > plen || tbf > tlen || tef > tlen) {
        if (t == 0) {
          p.status[pair] = kStInvalidForm;
          p.scores[pair] = 0;
          if (CIGAR) p.ops_len[pair] = 0;
          if (p.end_info) {
            p.end_info[3 * (int64_t)pair] = -1;
            p.end_info[3 * (int64_t)pair + 1] = -1;
            p.end_info[3 * (int64_t)pair + 2] = 0;
          }
        }
        group_sync<G>();
        continue;
      }
    }

    // ---- reset the rows the previous pair left non-NULL
    for (int r = 0; r < nrows; ++r) {
      const int2 mt = imeta[r];
      if (mt.x <= mt.y) null_range<OffT, G>(row(r), mt.x, mt.y, t, rb, g_pair);
    }
    group_sync<G>();
    for (int r = t; r < nrows; r += G) meta[r] = imeta[r] = make_int2(1, 0);

    // ---- stage sequences
    bool ok = (plen <= p.max_len) && (tlen <= p.max_len);
    if (ok) {
      ok &= stage_sequence<ENC, G>(p.seqs + p.p_off[pair], plen, P, t);
      ok &= stage_sequence<ENC, G>(p.seqs + p.t_off[pair], tlen, T, t);
    }
    if (!ok) {
      if (t == 0) {
        if (p.final_pass) {
          p.status[pair] = kStOOM;
          p.scores[pair] = 0;
          if (CIGAR) p.ops_len[pair] = 0;
        } else {
          p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
        }
      }
      group_sync<G>();
      continue;
    }

    // ---- score 0 (wavefront/wavefront_aligner.c:311-382): M[0][0] = 0, slot
    // 0, extended at once (every later M cell is extended as it is computed);
    // an alignment that begins in a gap component has offset 0 there and no M
    const int cb = p.comp_begin ? p.comp_begin[pair] : 0;
    const int ce = p.comp_end ? p.comp_end[pair] : 0;
    const int rowI1 = pen.R, rowD1 = pen.R + pen.RI1;
    const int rowI2 = pen.R + 2 * pen.RI1, rowD2 = rowI2 + pen.RI2;
    // ring row of component c for the current slots (cur1: I1/D1, cur2: I2/D2)
    auto comp_row = [&](int c, int cM, int c1, int c2) -> int {
      return c == 0 ? cM : c == 1 ? rowI1 + c1 : c == 2 ? rowD1 + c1 : c == 3 ? rowI2 + c2 : rowD2 + c2;
    };
    // ends-free with match 0: M[0] spans [-pattern_begin_free,
    // text_begin_free], diagonal k starting at (v,h) = (max(0,-k), max(0,k))
    // (wavefront/wavefront_aligner.c:250-305)
    const int e_lo = (EF && cb == 0 && pen.match == 0) ? -pbf : 0;
    const int e_hi = (EF && cb == 0 && pen.match == 0) ? tbf : 0;
    // the terminating diagonal of the last extended M wavefront (INT32_MAX:
    // none): ends-free, the first one that reaches an end within the free
    // lengths; end-to-end ending in M, k_end once its cell reaches (plen,
    // tlen) -- found by the cell loop, so no step re-reads the row
    int ef_k = INT32_MAX;
    const bool m_end = !EF && ce == 0;
    auto ef_done = [&](int off, int k) -> bool {
      const int vv = off - k;
      return (off >= tlen && plen - vv <= pef) || (vv >= plen && tlen - off <= tef);
    };
    if (EF && cb == 0) {
      int qk = INT32_MAX;
      for (int k = e_lo + t; k <= e_hi; k += G) {
        const int v0 = max(0, -k), h0 = max(0, k);
        const int off = h0 + lcp<ENC>(P, T, v0, h0, min(plen - v0, tlen - h0), nwords, g_pair);
        RING_ST(row(0), k, (OffT)off);
        if (ef_done(off, k)) qk = min(qk, k);
      }
      ef_k = gmin(qk);
      if (t == 0) {
        meta[0] = imeta[0] = make_int2(e_lo, e_hi);
        if (CIGAR) table[0] = BtRow{0, 0, 0};
      }
    } else {
      const int L0 = cb == 0 ? lcp<ENC>(P, T, 0, 0, min(plen, tlen), nwords, g_pair) : 0;
      if (m_end && cb == 0 && plen == tlen && L0 >= tlen) ef_k = 0;  // k_end == 0
      if (t == 0) {
        const int r0 = comp_row(cb, 0, 0, 0);
        RING_ST(row(r0), 0, (OffT)L0);
        meta[r0] = imeta[r0] = make_int2(0, 0);
        if (CIGAR) table[0] = BtRow{0, 0, 0};
      }
    }
    group_sync<G>();

    int s = 0;
    int curM = 0, cur1 = 0, cur2 = 0;  // ring slots of score s
    int null_steps = 0;
    // cut-off state as wavefront_heuristic_clear leaves it
    // (wavefront/wavefront_heuristic.c:114-121): wait counter, best SW score,
    // its diagonal (INT32_MAX: none yet), offset and WFA score
    int steps_wait = p.h_steps;
    int max_sw = 0, max_sw_k = INT32_MAX, max_wf = -1;
    int32_t max_sw_off = kNull;
    int64_t cursor = 0;  // choice bytes used (slice)
    int nblk = 0, cur_blk = -1;  // pool: blocks held, block being filled
    int64_t blk_off = 0, pool_used = 0;
    int result = 0;      // 1 done, -1 overflow, 2 max steps, 3 unreachable, 4 guard
    const int k_end = tlen - plen;
    int mlo = cb == 0 ? e_lo : 1, mhi = cb == 0 ? e_hi : 0;  // trimmed limits of M[s]
    bool m_exists = (cb == 0);

    while (true) {
      // ================= termination on the extended M[s], or on the end
      // component (wavefront/wavefront_termination.c:37-108); checked only
      // where M[s] exists (wavefront/wavefront_extend.c:93-106)
      if (m_exists) {
        if (EF || m_end) {
          // wavefront/wavefront_termination.c:37-60 (end-to-end: k_end's cell
          // is in M[s]'s limits and has reached tlen) and :115-162 (ends-free,
          // in extension order), as the cell loop found them
          if (ef_k != INT32_MAX) {
            result = 1;
            break;
          }
        } else {
          const int re = comp_row(ce, curM, cur1, cur2);
          const int2 em = meta[re];
          if (em.x <= k_end && k_end <= em.y && RING_LD(row(re), k_end) >= tlen) {
            result = 1;
            break;
          }
        }
      } else if (null_steps > pen.R) {
        // Edit and indel: the reference counts null steps only for a missing
        // wavefront (wavefront/wavefront_extend.c:93-101) and its edit driver
        // allocates every one, so null steps do not end it; no later cell can
        // be valid, and only the step limit does (wavefront/wavefront_
        // unialign.c:102-107).  Without a step limit it never ends: reported
        // unreachable here.
        result = (edit_like && p.max_steps != INT32_MAX) ? 2 : 3;
        break;
      }

      // ================= heuristic cut-off of the extended M[s]
      // (wavefront/wavefront_heuristic.c:506-563): one of wf-adaptive/wfmash,
      // one of x-drop/z-drop, one of banded static/adaptive, sharing one
      // wait counter.  Only the limits of M[s] (and, intersected, of its I/D
      // rows) shrink; the cut offsets stay in the rows' initialised windows.
      if (HEUR && m_exists && mlo <= mhi) {
        --steps_wait;
        const OffT* const mr = row(curM);
        const int hs = p.heur;
        int nlo = mlo, nhi = mhi;
        // wf-adaptive / wfmash (:229-289): cells further from the end than the
        // closest by more than max_distance_threshold, from both ends, keeping
        // the end diagonal's side
        if ((hs & (kHsWfadaptive | kHsWfmash)) && steps_wait <= 0 && nhi - nlo + 1 >= p.h_min_len) {
          const bool wm = !(hs & kHsWfadaptive);
          // wfmash weighs each side by its length (:134-145), in float as the
          // reference does
          const int mfactor = wm ? __float2int_rz(__fdiv_rn((float)(plen + tlen), 2.0f)) : 0;
          auto dist = [&](int k) -> int {
            const int32_t off = RING_LD(mr, k);
            if (off < 0) return 1 << 30;
            if (!wm) return max(plen - (off - k), tlen - off);
            const int lv = __float2int_rz(
                __fmul_rn(__fdiv_rn((float)(plen - (off - k)), (float)plen), (float)mfactor));
            const int lh = __float2int_rz(
                __fmul_rn(__fdiv_rn((float)(tlen - off), (float)tlen), (float)mfactor));
            return max(lv, lh);
          };
          int dmin = max(plen, tlen);
          for (int k = nlo + t; k <= nhi; k += G) dmin = min(dmin, dist(k));
          dmin = gmin(dmin);
          const int top = min(k_end, nhi);
          int first = INT32_MAX;
          for (int k = nlo + t; k < top; k += G)
            if (dist(k) - dmin <= p.h_max_dist) { first = k; break; }
          first = gmin(first);
          const int wlo = first == INT32_MAX ? max(nlo, top) : first;
          const int bot = max(k_end, wlo);
          int last = INT32_MIN;
          for (int k = nhi - t; k > bot; k -= G)
            if (dist(k) - dmin <= p.h_max_dist) { last = k; break; }
          last = gmax(last);
          nhi = last == INT32_MIN ? min(nhi, bot) : last;
          nlo = wlo;
          steps_wait = p.h_steps;
        }
        // x-drop (:326-380) / z-drop (:397-450) on the cells' SW scores
        // (wavefront/wavefront_penalties.h:73), with the first best cell
        if ((hs & (kHsXdrop | kHsZdrop)) && steps_wait <= 0) {
          const int swg = pen.match != 0 ? -pen.match : -1;
          auto sw = [&](int k, int32_t off) -> int { return (swg * (2 * off - k) - s) / 2; };
          int tbest = INT32_MIN, tk = INT32_MAX;
          int32_t toff = 0;
          for (int k = nlo + t; k <= nhi; k += G) {
            const int32_t off = RING_LD(mr, k);
            if (off < 0) continue;
            const int sc = sw(k, off);
            if (sc > tbest) { tbest = sc; tk = k; toff = off; }
          }
          const int cmax = gmax(tbest);
          int cmax_k = gmin(tbest == cmax ? tk : INT32_MAX);
          int32_t cmax_off = gmax(tk == cmax_k && tbest == cmax ? toff : INT32_MIN);
          if (cmax == INT32_MIN) { cmax_k = 0; cmax_off = 0; }
          bool dropped = false;
          if (hs & kHsXdrop) {
            if (max_sw_k != INT32_MAX) {
              // cells xdrop or more below the best seen are cut from both ends
              auto keep = [&](int k) -> bool {
                const int32_t off = RING_LD(mr, k);
                return off >= 0 && wsub32(max_sw, sw(k, off)) < p.h_xdrop;
              };
              int first = INT32_MAX;
              for (int k = nlo + t; k <= nhi; k += G)
                if (keep(k)) { first = k; break; }
              first = gmin(first);
              const int xlo = first == INT32_MAX ? nhi + 1 : first;
              int last = INT32_MIN;
              for (int k = nhi - t; k >= xlo; k -= G)
                if (keep(k)) { last = k; break; }
              last = gmax(last);
              if (xlo <= nhi) nhi = last;
              nlo = xlo;
              if (cmax > max_sw) { max_sw = cmax; max_sw_k = cmax_k; }
            } else {
              max_sw = cmax;
              max_sw_k = cmax_k;
            }
          } else if (max_sw_k != INT32_MAX) {
            if (cmax > max_sw) {
              max_sw = cmax; max_wf = s; max_sw_k = cmax_k; max_sw_off = cmax_off;
            } else if (wsub32(max_sw, cmax) > p.h_zdrop) {
              dropped = true;
            }
          } else {
            max_sw = cmax; max_wf = s; max_sw_k = cmax_k; max_sw_off = cmax_off;
          }
          if (dropped) {  // z-drop ends the alignment at the best cell seen
            result = 5;
            break;
          }
          steps_wait = p.h_steps;
        }
        // banded (:451-505)
        if (hs & kHsBandedStatic) {
          nlo = max(nlo, p.h_min_k);
          nhi = min(nhi, p.h_max_k);
        } else if ((hs & kHsBandedAdaptive) && steps_wait <= 0 && nhi - nlo + 1 >= 4) {
          const int len = nhi - nlo + 1, maxlen = p.h_max_k - p.h_min_k + 1;
          if (len > maxlen) {
            // place the band by the distances of four sampled cells
            auto dist = [&](int k) -> int {
              const int32_t off = RING_LD(mr, k);
              return off >= 0 ? max(plen - (off - k), tlen - off) : (1 << 30);
            };
            const int leeway = (len - maxlen) / 2, quarter = len / 4;
            int blo = nlo;
            if (dist(nlo) > dist(nhi)) blo += leeway;
            if (dist(nlo + quarter) > dist(nlo + 2 * quarter)) blo += leeway;
            nhi = min(blo + maxlen - 1, nhi);
            nlo = max(blo, nlo);
          }
          steps_wait = p.h_steps;
        }
        if (nlo != mlo || nhi != mhi) {
          if (EF && s == 0) {
            // the ends-free score-0 wavefront keeps the initialised window
            // [0,0] inside its limits; the first compute step NULL-pads from
            // beyond min/max(window, limits) (wavefront/wavefront_compute.c:
            // 498-527), so the cells cut here are NULLed, and a null row keeps
            // [0,0]
            const int2 ow = imeta[curM];
            const int wx = nlo <= nhi ? min(0, nlo) : 0, wy = nlo <= nhi ? max(0, nhi) : 0;
            OffT* const mw = row(curM);
            for (int k = ow.x + t; k < wx; k += G) RING_ST(mw, k, null_of<OffT>());
            for (int k = wy + 1 + t; k <= ow.y; k += G) RING_ST(mw, k, null_of<OffT>());
            group_sync<G>();
            if (t == 0) imeta[curM] = make_int2(wx, wy);
          }
          mlo = nlo;
          mhi = nhi;
          if (t == 0) {
            meta[curM] = make_int2(nlo, nhi);
            if (!lin) {  // one component: nothing to intersect (:549)
              const int nr = A2P ? 4 : 2;
              for (int j = 0; j < nr; ++j) {
                const int r = j == 0 ? rowI1 + cur1 : j == 1 ? rowD1 + cur1 : j == 2 ? rowI2 + cur2 : rowD2 + cur2;
                const int2 m = meta[r];
                meta[r] = make_int2(max(m.x, nlo), min(m.y, nhi));
              }
            }
          }
          group_sync<G>();
        }
      }

      // ================= compute score s+1
      ++s;
      if (s > p.table_cap) {  // above the reference's score bound: a guard, never hit
        result = 4;
        break;
      }
      curM = (curM + 1 == pen.R) ? 0 : curM + 1;
      cur1 = (cur1 + 1 == pen.RI1) ? 0 : cur1 + 1;
      if (A2P) cur2 = (cur2 + 1 == pen.RI2) ? 0 : cur2 + 1;

      // inputs (wavefront/wavefront_compute.c:306-352); score < 0 -> empty
      const int sMx = ring_back(curM, pen.x, pen.R);
      const int sMo1 = ring_back(curM, pen.o1 + pen.e1, pen.R);
      const int sI1 = ring_back(cur1, pen.e1, pen.RI1);
      const int2 kEmpty = make_int2(1, 0);
      const int2 eMx = (has_x && s - pen.x >= 0) ? meta[sMx] : kEmpty;
      const int2 eMo1 = (s - pen.o1 - pen.e1 >= 0) ? meta[sMo1] : kEmpty;
      const int2 eI1 = (!lin && s - pen.e1 >= 0) ? meta[rowI1 + sI1] : kEmpty;
      const int2 eD1 = (!lin && s - pen.e1 >= 0) ? meta[rowD1 + sI1] : kEmpty;
      int sMo2 = 0, sI2 = 0;
      int2 eMo2 = kEmpty, eI2 = kEmpty, eD2 = kEmpty;
      if (A2P) {
        sMo2 = ring_back(curM, pen.o2 + pen.e2, pen.R);
        sI2 = ring_back(cur2, pen.e2, pen.RI2);
        if (s - pen.o2 - pen.e2 >= 0) eMo2 = meta[sMo2];
        if (s - pen.e2 >= 0) {
          eI2 = meta[rowI2 + sI2];
          eD2 = meta[rowD2 + sI2];
        }
      }
      const bool vMx = eMx.x <= eMx.y, vMo1 = eMo1.x <= eMo1.y;
      const bool vI1 = eI1.x <= eI1.y, vD1 = eD1.x <= eD1.y;
      const bool vMo2 = A2P && eMo2.x <= eMo2.y;
      const bool vI2 = A2P && eI2.x <= eI2.y, vD2 = A2P && eD2.x <= eD2.y;

      OffT* const oM = row(curM);
      OffT* const oI1 = row(rowI1 + cur1);
      OffT* const oD1 = row(rowD1 + cur1);
      OffT* const oI2 = A2P ? row(rowI2 + cur2) : nullptr;
      OffT* const oD2 = A2P ? row(rowD2 + cur2) : nullptr;
      // what a reused slot holds: its initialised window
      const int2 oldM = imeta[curM], oldI1 = imeta[rowI1 + cur1], oldD1 = imeta[rowD1 + cur1];
      const int2 oldI2 = A2P ? imeta[rowI2 + cur2] : kEmpty;
      const int2 oldD2 = A2P ? imeta[rowD2 + cur2] : kEmpty;

      // ends-free with match < 0: the begin cells (0,ek) and (ek,0) enter at
      // the scores that are multiples of -match, ek = s / -match
      // (wavefront/wavefront_compute.c:124-262); INT32_MIN: none
      int ekT = INT32_MIN, ekP = INT32_MIN;
      if (EF && pen.match != 0 && cb == 0 && (pbf > 0 || tbf > 0) && s % (-pen.match) == 0) {
        const int ek = s / (-pen.match);
        if (tbf >= ek) ekT = ek;
        if (pbf >= ek) ekP = -ek;
      }
      const bool inject = EF && (ekT != INT32_MIN || ekP != INT32_MIN);
      const bool all_null = !(vMx | vMo1 | vI1 | vD1 | vMo2 | vI2 | vD2);

      // wavefront/wavefront_compute_affine.c:236-243: all inputs null -> null
      // step (with begin cells to enter, an M wavefront of those)
      if (all_null && !inject) {
        ++null_steps;
        // Exact runs read a row only within its limits, so a null step just
        // empties the limits of the slots it takes over; they keep their old
        // window, which the slot's next write (or the next pair) clears.
        // Under the heuristic the windows are read too: clear them now.
        if (HEUR) {
          clear_outside<OffT, G>(oM, oldM, 1, 0, t, rb, g_pair);
          clear_outside<OffT, G>(oI1, oldI1, 1, 0, t, rb, g_pair);
          clear_outside<OffT, G>(oD1, oldD1, 1, 0, t, rb, g_pair);
          if (A2P) {
            clear_outside<OffT, G>(oI2, oldI2, 1, 0, t, rb, g_pair);
            clear_outside<OffT, G>(oD2, oldD2, 1, 0, t, rb, g_pair);
          }
          group_sync<G>();
        }
        if (t == 0) {
          meta[curM] = kEmpty;
          meta[rowI1 + cur1] = kEmpty;
          meta[rowD1 + cur1] = kEmpty;
          if (A2P) {
            meta[rowI2 + cur2] = kEmpty;
            meta[rowD2 + cur2] = kEmpty;
          }
          if (HEUR) {
            imeta[curM] = imeta[rowI1 + cur1] = imeta[rowD1 + cur1] = kEmpty;
            if (A2P) imeta[rowI2 + cur2] = imeta[rowD2 + cur2] = kEmpty;
          }
        }
        if (CIGAR) {
          if (s >= p.table_cap) {
            result = -1;
            break;
          }
          if (t == 0 && CHK(s < p.table_cap, 32, s)) table[s] = BtRow{-1, 0, -1};
        }
        group_sync<G>();
        m_exists = false;
        if (s >= p.max_steps) {
          result = 2;
          break;
        }
        continue;
      }
      if (all_null) ++null_steps;  // the begin cells alone (:382-407)
      else null_steps = 0;

      // wavefront/wavefront_compute.c:40-87: output range
      int lo = INT32_MAX, hi = INT32_MIN;
      if (HEUR && !edit_like) {
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
      // begin cells beyond the computed range [lo0,hi0] widen it on their
      // side, with NULL cells between (wavefront/wavefront_compute.c:173-262);
      // a step whose inputs are all null computes no cell
      const int lo0 = all_null ? INT32_MAX : lo, hi0 = all_null ? INT32_MIN : hi;
      if (inject) {
        if (all_null) {
          lo = min(ekP != INT32_MIN ? ekP : ekT, ekT != INT32_MIN ? ekT : ekP);
          hi = max(ekP != INT32_MIN ? ekP : ekT, ekT != INT32_MIN ? ekT : ekP);
        } else {
          if (ekP != INT32_MIN) lo = min(lo, ekP);
          if (ekT != INT32_MIN) hi = max(hi, ekT);
        }
      }
      const int width = hi - lo + 1;
      if (CIGAR && (s >= p.table_cap || (!pooled && cursor + width > p.bits_cap))) {
        result = -1;
        break;
      }
      int64_t bpos = cursor;  // this row's first choice byte in the store
      if (pooled) {
        if (pool_used + width > p.pair_cap) {  // over the pair's back-trace budget
          result = -1;
          break;
        }
        pool_used += width;
        if (cur_blk < 0 || blk_off + width > p.block_bytes) {
          int b = -1;
          if (nblk < p.max_blocks && t == 0) b = pool_pop(p);
          b = gbcast(b);
          if (b < 0) {  // pool empty: a later pass retries the pair
            result = -1;
            break;
          }
          if (t == 0) owned[nblk] = b;
          ++nblk;
          cur_blk = b;
          blk_off = 0;
        }
        bpos = (int64_t)cur_blk * p.block_bytes + blk_off;
      }
      clear_outside<OffT, G>(oM, oldM, lo, hi, t, rb, g_pair);
      clear_outside<OffT, G>(oI1, oldI1, lo, hi, t, rb, g_pair);
      clear_outside<OffT, G>(oD1, oldD1, lo, hi, t, rb, g_pair);
      if (A2P) {
        clear_outside<OffT, G>(oI2, oldI2, lo, hi, t, rb, g_pair);
        clear_outside<OffT, G>(oD2, oldD2, lo, hi, t, rb, g_pair);
      }
      // clears and the cells below touch disjoint elements: no CTA barrier
      if (G == 32) __syncwarp();

      const OffT* const rMx = vMx ? row(sMx) : null_row;
      const OffT* const rMo1 = vMo1 ? row(sMo1) : null_row;
      const OffT* const rI1 = vI1 ? row(rowI1 + sI1) : null_row;
      const OffT* const rD1 = vD1 ? row(rowD1 + sI1) : null_row;
      const OffT* const rMo2 = vMo2 ? row(sMo2) : null_row;
      const OffT* const rI2 = vI2 ? row(rowI2 + sI2) : null_row;
      const OffT* const rD2 = vD2 ? row(rowD2 + sI2) : null_row;
      // The reference's back-trace reads an input within its initialised
      // window even when the row is null (wavefront/wavefront_backtrace.c:
      // 63-219), while the compute step reads the all-NULL row: the two
      // differ only for a row that a cut-off left with empty limits and a
      // non-empty window.  Choice bytes then follow the back-trace.
      auto window_row = [&](bool valid, int r, int score_back) -> const OffT* {
        if (valid || score_back < 0) return nullptr;
        const int2 w = imeta[r];
        return w.x <= w.y ? row(r) : nullptr;
      };
      const OffT* wI1 = nullptr;
      const OffT* wD1 = nullptr;
      const OffT* wI2 = nullptr;
      const OffT* wD2 = nullptr;
      if (CIGAR && HEUR && !lin) {
        wI1 = window_row(vI1, rowI1 + sI1, s - pen.e1);
        wD1 = window_row(vD1, rowD1 + sI1, s - pen.e1);
        if (A2P) {
          wI2 = window_row(vI2, rowI2 + sI2, s - pen.e2);
          wD2 = window_row(vD2, rowD2 + sI2, s - pen.e2);
        }
      }
      const OffT* wMx = nullptr;
      const OffT* wMo1 = nullptr;
      const OffT* wMo2 = nullptr;
      if (CIGAR && HEUR) {
        if (has_x) wMx = window_row(vMx, sMx, s - pen.x);
        wMo1 = window_row(vMo1, sMo1, s - pen.o1 - pen.e1);
        if (A2P) wMo2 = window_row(vMo2, sMo2, s - pen.o2 - pen.e2);
      }
      const bool ghost = wI1 || wD1 || wI2 || wD2 || wMx || wMo1 || wMo2;
      uint8_t* const brow = CIGAR ? bt + bpos - lo : nullptr;
      // edit and indel NULL the two elements beyond each end of M[s-1]
      // (wavefront/wavefront_compute_edit.c:352-356): cells a cut-off left in
      // the initialised window are the only ones that can hold values there
      if (HEUR && edit_like && vMo1) {
        const int2 w = imeta[sMo1];
        OffT* const r = row(sMo1);
        if (t == 0) {
          const int ks[4] = {eMo1.x - 2, eMo1.x - 1, eMo1.y + 1, eMo1.y + 2};
          for (int j = 0; j < 4; ++j)
            if (ks[j] >= w.x && ks[j] <= w.y) RING_ST(r, ks[j], null_of<OffT>());
        }
        group_sync<G>();
      }

      int tloM = INT32_MAX, thiM = INT32_MIN;
      int tloI1 = INT32_MAX, thiI1 = INT32_MIN, tloD1 = INT32_MAX, thiD1 = INT32_MIN;
      int tloI2 = INT32_MAX, thiI2 = INT32_MIN, tloD2 = INT32_MAX, thiD2 = INT32_MIN;
      int qk = INT32_MAX;  // ends-free: first terminating diagonal of this thread
      int wmin = INT32_MAX;  // edit pruning: best worst case over the unextended cells
      // Software-pipelined: the next cell's inputs are loaded before the
      // current cell is computed, so one load latency overlaps the work.
      int32_t n_mo1_m = 0, n_mo1_p = 0, n_i1_e = 0, n_d1_e = 0, n_mx = 0;
      int32_t n_mo2_m = 0, n_mo2_p = 0, n_i2_e = 0, n_d2_e = 0;
      auto load_inputs = [&](int kk) {
        n_mo1_m = RING_LD(rMo1, kk - 1);
        n_mo1_p = RING_LD(rMo1, kk + 1);
        n_i1_e = RING_LD(rI1, kk - 1);
        n_d1_e = RING_LD(rD1, kk + 1);
        n_mx = RING_LD(rMx, kk);
        if (A2P) {
          n_mo2_m = RING_LD(rMo2, kk - 1);
          n_mo2_p = RING_LD(rMo2, kk + 1);
          n_i2_e = RING_LD(rI2, kk - 1);
          n_d2_e = RING_LD(rD2, kk + 1);
        }
      };
      if (lo + t <= hi) load_inputs(lo + t);
      for (int k = lo + t; k <= hi; k += G) {
        const int32_t mo1_m = n_mo1_m, mo1_p = n_mo1_p, i1_e = n_i1_e, d1_e = n_d1_e, mx = n_mx;
        const int32_t mo2_m = n_mo2_m, mo2_p = n_mo2_p, i2_e = n_i2_e, d2_e = n_d2_e;
        if (k + G <= hi) load_inputs(k + G);
        // wavefront/wavefront_compute_affine.c:66-84
        int32_t i1 = max(mo1_m, i1_e) + 1;
        int32_t d1 = max(mo1_p, d1_e);
        const int32_t mis = mx + 1;
        int32_t ins = i1, del = d1;
        int32_t i2 = kNull, d2 = kNull;
        if (A2P) {
          // wavefront/wavefront_compute_affine2p.c:78-95
          i2 = max(mo2_m, i2_e) + 1;
          d2 = max(mo2_p, d2_e);
          ins = max(i1, i2);
          del = max(d1, d2);
        }
        int32_t best = max(del, max(mis, ins));
        if (inject && (k < lo0 || k > hi0)) {  // not computed: NULL
          i1 = d1 = i2 = d2 = best = null_of<OffT>();
        }
        bool okM = in_bounds(best, k, plen, tlen);
        // a begin cell replaces a computed one that does not lie ahead of it
        bool begin_cell = false;
        if (inject && (k == ekT || k == ekP)) {
          const int32_t bo = k > 0 ? k : 0;  // offset of (0,k) or (-k,0)
          if ((okM ? best : kNull) <= bo) {
            best = bo;
            okM = true;
            begin_cell = true;
          }
        }
        // Trim tests (wavefront/wavefront_compute.c:579-613), simplified: a
        // non-NULL insertion keeps its source's v <= plen, a deletion its h <= tlen
        const bool okI1 = (uint32_t)i1 <= (uint32_t)tlen;
        const bool okD1 = (uint32_t)(d1 - k) <= (uint32_t)plen;
        // insertion values drift upwards from NULL: keep narrow NULLs canonical
        if (sizeof(OffT) == 2 && i1 < 0) i1 = null_of<OffT>();
        // extend the new M cell now (wavefront/wavefront_extend.c:86-121): the
        // reference extends M[s] right after computing it, before score s+1
        int32_t mext = null_of<OffT>();
        if (okM) {
          const int v = best - k;
          if (prune) wmin = min(wmin, max(plen - v, tlen - best));
          mext = best + lcp<ENC>(P, T, v, best, min(plen - v, tlen - best), nwords, g_pair);
          if (EF && ef_done(mext, k)) qk = min(qk, k);
          if (m_end && k == k_end && mext >= tlen) qk = k;
        }
        RING_ST(oM, k, (OffT)mext);
        RING_ST(oI1, k, (OffT)i1);
        RING_ST(oD1, k, (OffT)d1);
        if (okM) { tloM = min(tloM, k); thiM = k; }
        if (okI1) { tloI1 = min(tloI1, k); thiI1 = k; }
        if (okD1) { tloD1 = min(tloD1, k); thiD1 = k; }
        if (A2P) {
          const bool okI2 = (uint32_t)i2 <= (uint32_t)tlen;
          const bool okD2 = (uint32_t)(d2 - k) <= (uint32_t)plen;
          if (sizeof(OffT) == 2 && i2 < 0) i2 = null_of<OffT>();
          RING_ST(oI2, k, (OffT)i2);
          RING_ST(oD2, k, (OffT)d2);
          if (okI2) { tloI2 = min(tloI2, k); thiI2 = k; }
          if (okD2) { tloD2 = min(tloD2, k); thiD2 = k; }
        }
        if (CIGAR) {
          // M source with the reference's tie order: mismatch > D2 > D1 > I2 > I1
          uint8_t c;
          if (mis == best) c = kSrcX;
          else if (A2P && d2 == best) c = kSrcD2;
          else if (d1 == best) c = kSrcD1;
          else if (A2P && i2 == best) c = kSrcI2;
          else c = kSrcI1;
          if (!lin) {  // one component: every gap opens from M
            c |= (uint8_t)(i1_e >= mo1_m) << 3;
            c |= (uint8_t)(d1_e >= mo1_p) << 4;
          }
          if (A2P) {
            c |= (uint8_t)(i2_e >= mo2_m) << 5;
            c |= (uint8_t)(d2_e >= mo2_p) << 6;
          }
          if (HEUR && ghost) {
            // back-trace candidates with the cut rows' window values
            const int32_t gmis = wMx ? RING_LD(wMx, k) + 1 : mis;
            const int32_t gmo1m = wMo1 ? RING_LD(wMo1, k - 1) : mo1_m;
            const int32_t gmo1p = wMo1 ? RING_LD(wMo1, k + 1) : mo1_p;
            const int32_t wi1e = wI1 ? RING_LD(wI1, k - 1) : i1_e;
            const int32_t wd1e = wD1 ? RING_LD(wD1, k + 1) : d1_e;
            const int32_t wi1 = max(gmo1m, wi1e) + 1, wd1 = max(gmo1p, wd1e);
            int32_t wi2 = kNull, wd2 = kNull, wi2e = i2_e, wd2e = d2_e;
            int32_t gmo2m = mo2_m, gmo2p = mo2_p;
            if (A2P) {
              gmo2m = wMo2 ? RING_LD(wMo2, k - 1) : mo2_m;
              gmo2p = wMo2 ? RING_LD(wMo2, k + 1) : mo2_p;
              wi2e = wI2 ? RING_LD(wI2, k - 1) : i2_e;
              wd2e = wD2 ? RING_LD(wD2, k + 1) : d2_e;
              wi2 = max(gmo2m, wi2e) + 1;
              wd2 = max(gmo2p, wd2e);
            }
            const int32_t wbest = max(max(wd1, wd2), max(gmis, max(wi1, wi2)));
            if (gmis == wbest) c = kSrcX;
            else if (A2P && wd2 == wbest) c = kSrcD2;
            else if (wd1 == wbest) c = kSrcD1;
            else if (A2P && wi2 == wbest) c = kSrcI2;
            else c = kSrcI1;
            if (!lin) {
              c |= (uint8_t)(wi1e >= gmo1m) << 3;
              c |= (uint8_t)(wd1e >= gmo1p) << 4;
            }
            if (A2P) {
              c |= (uint8_t)(wi2e >= gmo2m) << 5;
              c |= (uint8_t)(wd2e >= gmo2p) << 6;
            }
          }
          if (EF && begin_cell) c = kBegin;  // the walk stops here
          if (CHK(pooled || cursor + (k - lo) < p.bits_cap, 30, cursor + (k - lo))) brow[k] = c;
        }
      }
      if (G == 32) __syncwarp();
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
      if (EF || m_end) qk = __reduce_min_sync(kFull, qk);
      if (prune) wmin = __reduce_min_sync(kFull, wmin);
      if (G > 32) {
        // across the group's warps: one barrier; the partials are next
        // written after the end-of-step barrier, so they need no second one
        int32_t* const pr = gred + wig * kRedVals;
        if (lane == 0) {
          pr[0] = tloM; pr[1] = thiM; pr[2] = tloI1; pr[3] = thiI1; pr[4] = tloD1; pr[5] = thiD1;
          if (A2P) { pr[6] = tloI2; pr[7] = thiI2; pr[8] = tloD2; pr[9] = thiD2; }
          if (EF || m_end) pr[10] = qk;
          if (prune) pr[11] = wmin;
        }
        __syncthreads();
        for (int w = 0; w < G / 32; ++w) {
          const int32_t* const q = gred + w * kRedVals;
          tloM = min(tloM, q[0]); thiM = max(thiM, q[1]);
          tloI1 = min(tloI1, q[2]); thiI1 = max(thiI1, q[3]);
          tloD1 = min(tloD1, q[4]); thiD1 = max(thiD1, q[5]);
          if (A2P) {
            tloI2 = min(tloI2, q[6]); thiI2 = max(thiI2, q[7]);
            tloD2 = min(tloD2, q[8]); thiD2 = max(thiD2, q[9]);
          }
          if (EF || m_end) qk = min(qk, q[10]);
          if (prune) wmin = min(wmin, q[11]);
        }
      }
      if (EF || m_end) ef_k = qk;
      if (prune && thiM - tloM + 1 >= 1000) {
        // exact pruning of a wide end-to-end edit wavefront on its unextended
        // offsets (wavefront/wavefront_compute_edit.c:220-279): a diagonal's
        // best case is |k - k_end| edits, its worst the larger remainder;
        // diagonals whose best exceeds the least worst are dropped
        const int sk = tloM + (thiM - tloM) / 2;
        int32_t so = max(RING_LD(rMo1, sk + 1), max(RING_LD(rMx, sk), RING_LD(rMo1, sk - 1)) + 1);
        if (!in_bounds(so, sk, plen, tlen)) so = -1;
        if (so >= 0) {
          const int smax = max(plen - (so - sk), tlen - so);
          if (!(abs(tloM - k_end) <= smax && abs(thiM - k_end) <= smax)) {
            const int a = max(tloM, k_end - wmin);
            const int nlo = (a <= min(thiM, k_end + wmin)) ? a : thiM + 1;
            const int b = min(thiM, k_end + wmin);
            const int nhi = (b > nlo && b >= k_end - wmin) ? b : nlo;
            tloM = nlo;
            thiM = nhi;
          }
        }
      }
      trim_fill<OffT, G>(oM, lo, hi, tloM, thiM, t, rb, g_pair);
      trim_fill<OffT, G>(oI1, lo, hi, tloI1, thiI1, t, rb, g_pair);
      trim_fill<OffT, G>(oD1, lo, hi, tloD1, thiD1, t, rb, g_pair);
      if (A2P) {
        trim_fill<OffT, G>(oI2, lo, hi, tloI2, thiI2, t, rb, g_pair);
        trim_fill<OffT, G>(oD2, lo, hi, tloD2, thiD2, t, rb, g_pair);
      }
      if (G == 32) __syncwarp();
      if (t == 0) {
        meta[curM] = imeta[curM] = make_int2(tloM, thiM);
        meta[rowI1 + cur1] = imeta[rowI1 + cur1] = make_int2(tloI1, thiI1);
        meta[rowD1 + cur1] = imeta[rowD1 + cur1] = make_int2(tloD1, thiD1);
        if (A2P) {
          meta[rowI2 + cur2] = imeta[rowI2 + cur2] = make_int2(tloI2, thiI2);
          meta[rowD2 + cur2] = imeta[rowD2 + cur2] = make_int2(tloD2, thiD2);
        }
        if (CIGAR && CHK(s < p.table_cap, 31, s)) table[s] = BtRow{bpos, lo, width};
      }
      if (CIGAR) {
        if (pooled) blk_off += width;
        else cursor += width;
      }
      mlo = tloM;
      mhi = thiM;
      m_exists = true;
      group_sync<G>();
      // wavefront/wavefront_unialign.c:102-107
      if (s >= p.max_steps) {
        result = 2;
        break;
      }
    }

    // pool blocks go back when the pair is finished (every path below)
    auto release_blocks = [&]() {
      if (pooled && nblk > 0) {
        group_sync<G>();
        if (t == 0) pool_push(p, owned, nblk);
        nblk = 0;
        group_sync<G>();
      }
    };

    // classic score (wavefront/wavefront_compute.c:108-120), in the
    // reference's wrapping int arithmetic
    auto classic = [&](int ev, int eh) -> int {
      if (edit_like) return s;  // the distance itself
      if (pen.match == 0) return -s;
      return (int)((uint32_t)(-pen.match) * ((uint32_t)ev + (uint32_t)eh) - (uint32_t)s) / 2;
    };
    // ================= finish the pair (warp-uniform from here on)
    if (result != 1 && result != 5) {
      release_blocks();
      if (t == 0) {
        if (result == -1 && !p.final_pass) {
          p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
        } else {
          int st, sc, ev = -1, eh = -1;
          if (result == -1) { st = kStOOM; sc = 0; }
          else if (result == 2) { st = kStMaxSteps; sc = -p.max_steps; }
          else if (result == 3) {
            // the end unreachable (wavefront/wavefront_unialign.c:147-237) with
            // no end position (DPMATRIX_DIAGONAL_NULL, WAVEFRONT_OFFSET_NULL):
            // score-only reports the classic score there; a full run has no
            // CIGAR to trim, which leaves the cleared one
            st = kStPartial;
            if (CIGAR) {
              sc = INT32_MIN;
            } else {
              eh = kNull;
              ev = wsub32(kNull, INT32_MAX);
              sc = classic(ev, eh);
            }
          }
          else { st = kStUnattainable; sc = 0; }
          p.status[pair] = st;
          p.scores[pair] = sc;
          if (CIGAR) p.ops_len[pair] = 0;
          if (p.end_info) {
            p.end_info[3 * (int64_t)pair] = ev;
            p.end_info[3 * (int64_t)pair + 1] = eh;
            p.end_info[3 * (int64_t)pair + 2] = s;
          }
        }
      }
      group_sync<G>();
      continue;
    }
    // the end position: (plen, tlen) end-to-end, the terminating diagonal's
    // cell ends-free, the best cell seen when z-dropped
    // (wf_aligner->alignment_end_pos)
    const bool zdrop = HEUR && result == 5;
    int end_k = k_end, end_v = plen, end_h = tlen;
    if (zdrop) {
      end_k = max_sw_k;
      end_h = max_sw_off;
      end_v = end_h - end_k;
    } else if (EF) {
      end_k = ef_k;
      end_h = RING_LD(row(curM), ef_k);
      end_v = end_h - ef_k;
    }
    // a score-only run reports the classic score for the whole sequences
    // (wavefront/wavefront_unialign.c:160-165), a full run for the end position
    const int score = (CIGAR || zdrop) ? classic(end_v, end_h) : classic(plen, tlen);
    if (!CIGAR) {
      if (t == 0) {
        p.scores[pair] = score;
        p.status[pair] = zdrop ? kStPartial : kStCompleted;
        if (p.end_info) {
          p.end_info[3 * (int64_t)pair] = zdrop ? end_v : plen;
          p.end_info[3 * (int64_t)pair + 1] = zdrop ? end_h : tlen;
          p.end_info[3 * (int64_t)pair + 2] = s;
        }
      }
      group_sync<G>();
      continue;
    }

    // ================= back-trace over choice bytes (uniform walk), then a
    // forward replay that re-extends the matches of every M visit
    uint8_t* const items = pooled ? bits + owned_bytes : bits + cursor;
    const int64_t items_cap = pooled ? p.bits_cap - owned_bytes : p.bits_cap - cursor;
    int64_t n = 0;
    bool bad = false;
    bool items_full = false;  // walk items did not fit the back-trace slice
    int k_begin = 0;          // diagonal of the score-0 cell the walk reaches
    // z-drop: the walk starts at the best cell's diagonal from the current
    // score, where the current wavefront may hold no cell; the reference then
    // reads the sources' windows (wavefront/wavefront_backtrace.c:62-219), or,
    // finding none, writes the beginning as matches and gaps (:505-516)
    bool zfirst = zdrop, znosrc = false;
    if (G == 32 || wig == 0) {
      int st = ce;  // 0 M, 1 I1, 2 D1, 3 I2, 4 D2
      int ss = s, kk = end_k;
      while (true) {
        if (n + 2 > items_cap) { items_full = true; break; }
        if (ss < 0) { bad = true; break; }
        if (st == 0) {
          if (lane == 0 && CHK(n < items_cap, 33, n)) items[n] = 'E';
          ++n;
          if (ss == 0) {
            // ends-free: any diagonal of the score-0 wavefront
            bad = EF ? (kk < e_lo || kk > e_hi) : ((kk != 0) || (cb != 0));
            k_begin = kk;
            break;
          }
        } else if (ss == 0) {
          // the score-0 cell of an alignment that begins in a gap component
          bad = (kk != 0) || (st != cb);
          break;
        }
        if (!CHK(ss < p.table_cap, 34, ss)) { bad = true; break; }
        const BtRow te = table[ss];
        if (zfirst) {
          zfirst = false;
          // The reference's walk runs while v > 0 and h > 0
          // (wavefront/wavefront_backtrace.c:358): from a best cell on
          // the first row or column it takes no step, and its CIGAR is the
          // end gaps alone.
          if (end_v <= 0 || end_h <= 0) break;
          // The first step always takes the reference's candidates from the
          // sources: the best cell's diagonal may hold no cell at this score,
          // or an out-of-bounds one whose choice byte compares NULL inputs.
          {
            // candidates as the reference packs them: (offset << 4) | type,
            // larger wins (wavefront/wavefront_backtrace.c:36-59)
            auto cand = [&](int back, int r, int k, int add, int type) -> int64_t {
              if (ss - back < 0) return (int64_t)kNull;
              const int2 w = imeta[r];
              if (k < w.x || k > w.y) return (int64_t)kNull;
              return ((int64_t)(RING_LD(row(r), k) + add) << 4) | type;
            };
            int64_t best = has_x ? cand(pen.x, ring_back(curM, pen.x, pen.R), kk, 1, 9) : kNull;
            const int rMo1 = ring_back(curM, pen.o1 + pen.e1, pen.R);
            best = max(best, cand(pen.o1 + pen.e1, rMo1, kk - 1, 1, 1));
            best = max(best, cand(pen.o1 + pen.e1, rMo1, kk + 1, 0, 5));
            if (!lin) {
              const int s1 = ring_back(cur1, pen.e1, pen.RI1);
              best = max(best, cand(pen.e1, rowI1 + s1, kk - 1, 1, 2));
              best = max(best, cand(pen.e1, rowD1 + s1, kk + 1, 0, 6));
            }
            if (A2P) {
              const int rMo2 = ring_back(curM, pen.o2 + pen.e2, pen.R);
              const int s2 = ring_back(cur2, pen.e2, pen.RI2);
              best = max(best, cand(pen.o2 + pen.e2, rMo2, kk - 1, 1, 3));
              best = max(best, cand(pen.o2 + pen.e2, rMo2, kk + 1, 0, 7));
              best = max(best, cand(pen.e2, rowI2 + s2, kk - 1, 1, 4));
              best = max(best, cand(pen.e2, rowD2 + s2, kk + 1, 0, 8));
            }
            if (best < 0) { znosrc = true; break; }
            char op;
            switch ((int)(best & 15)) {
              case 9: op = 'X'; ss -= pen.x; break;
              case 1: op = 'I'; kk -= 1; ss -= pen.o1 + pen.e1; break;
              case 2: op = 'I'; kk -= 1; ss -= pen.e1; st = 1; break;
              case 3: op = 'I'; kk -= 1; ss -= pen.o2 + pen.e2; break;
              case 4: op = 'I'; kk -= 1; ss -= pen.e2; st = 3; break;
              case 5: op = 'D'; kk += 1; ss -= pen.o1 + pen.e1; break;
              case 6: op = 'D'; kk += 1; ss -= pen.e1; st = 2; break;
              case 7: op = 'D'; kk += 1; ss -= pen.o2 + pen.e2; break;
              default: op = 'D'; kk += 1; ss -= pen.e2; st = 4; break;
            }
            if (lane == 0 && CHK(n < items_cap, 36, n)) items[n] = (uint8_t)op;
            ++n;
            continue;
          }
        }
        if (te.width <= 0 || kk < te.lo || kk - te.lo >= te.width) { bad = true; break; }
        const int64_t bi = te.pos + (kk - te.lo);
        if (!CHK(pooled || (bi >= 0 && bi < p.bits_cap), 35, bi)) { bad = true; break; }
        const uint8_t c = bt[bi];
        char op = 0;
        if (EF && st == 0 && c == kBegin) {
          // a begin cell entered at this score (ends-free, match < 0): the
          // free beginning is written by the replay
          k_begin = kk;
          break;
        }
        if (st == 0) {
          const int src = c & 7;
          if (src == kSrcX) { op = 'X'; ss -= pen.x; }
          else if (src == kSrcD1) st = 2;
          else if (src == kSrcI1) st = 1;
          else if (src == kSrcD2) st = 4;
          else st = 3;
        } else if (st == 1) {
          op = 'I'; kk -= 1;
          if (c & 8) ss -= pen.e1; else { ss -= pen.o1 + pen.e1; st = 0; }
        } else if (st == 2) {
          op = 'D'; kk += 1;
          if (c & 16) ss -= pen.e1; else { ss -= pen.o1 + pen.e1; st = 0; }
        } else if (st == 3) {
          op = 'I'; kk -= 1;
          if (c & 32) ss -= pen.e2; else { ss -= pen.o2 + pen.e2; st = 0; }
        } else {
          op = 'D'; kk += 1;
          if (c & 64) ss -= pen.e2; else { ss -= pen.o2 + pen.e2; st = 0; }
        }
        if (op) {
          if (lane == 0 && CHK(n < items_cap, 36, n)) items[n] = (uint8_t)op;
          ++n;
        }
      }
    }
    group_sync<G>();
    if (G > 32) items_full = gbcast(items_full);
    release_blocks();  // the walk has read every choice byte it needs
    if (items_full) {
      // the same overflow as a full cell table: retry with a larger slice, or
      // WF_STATUS_OOM in the final pass
      if (t == 0) {
        if (!p.final_pass) {
          p.retry_items[atomicAdd(p.retry_count, 1)] = pair;
        } else {
          p.status[pair] = kStOOM;
          p.scores[pair] = 0;
          p.ops_len[pair] = 0;
        }
      }
      group_sync<G>();
      continue;
    }
    int out_n = 0;
    int fin_status = kStCompleted, fin_score = score, fin_v = end_v, fin_h = end_h;
    if ((G == 32 || wig == 0) && !bad) {
      uint8_t* const out = p.ops + p.ops_off[pair];
      int v = 0, h = 0;
      if (EF && k_begin != 0) {
        // a free beginning: insertions of the text's first k, or deletions of
        // the pattern's first -k (wavefront/wavefront_backtrace.c:506-516)
        const int nb = k_begin > 0 ? k_begin : -k_begin;
        const uint8_t op = k_begin > 0 ? 'I' : 'D';
        for (int j = lane; j < nb; j += 32)
          if (CHK(j < plen + tlen, 39, j)) out[j] = op;
        out_n = nb;
        v = max(0, -k_begin);
        h = max(0, k_begin);
      }
      int pops = 0;  // z-drop: trailing gaps the first match count takes back
      if (znosrc) {
        // no source at the best cell: insertions, deletions, then the
        // matches up to it (wavefront/wavefront_backtrace.c:505-516)
        const int mn = min(end_v, end_h), ni0 = end_h - mn, nd0 = end_v - mn;
        for (int j = lane; j < ni0 + nd0 + mn; j += 32)
          if (CHK(j < plen + tlen, 41, j)) out[j] = j < ni0 ? 'I' : (j < ni0 + nd0 ? 'D' : 'M');
        out_n = ni0 + nd0 + mn;
        v = end_v;
        h = end_h;
      }
      for (int64_t i = znosrc ? -1 : n - 1; i >= 0; --i) {
        const uint8_t it = items[i];
        if (it == 'E') {
          int L;
          if (zdrop && i == 0) {
            // the walk began at the best cell's diagonal from the current
            // score: the reference counts the matches up to the best cell's
            // offset without reading the sequences, and a negative count
            // takes back that many of the gaps it wrote to the ends first
            // (wavefront/wavefront_backtrace.c:76-100, :339-356)
            L = max(0, end_h - h);
            pops = max(0, h - end_h);
          } else {
            // a z-dropped trace can run past an end (the reference does not
            // check): no matches there
            L = lcp<ENC>(P, T, v, h, max(0, min(plen - v, tlen - h)), nwords, g_pair);
          }
          if (out_n + L > plen + tlen) { bad = true; break; }
          for (int j = lane; j < L; j += 32)
            if (CHK(out_n + j < plen + tlen, 37, out_n + j)) out[out_n + j] = 'M';
          out_n += L;
          v += L;
          h += L;
        } else {
          if (it == 'X') { bad = (v >= plen || h >= tlen); ++v; ++h; }
          else if (it == 'I') { bad = (h >= tlen); ++h; }
          else { bad = (v >= plen); ++v; }
          // the reference writes a z-dropped trace's operations past an end
          // as they come; its trim decides
          if (zdrop) bad = out_n >= plen + tlen;
          if (bad) break;
          if (lane == 0 && CHK(out_n < plen + tlen, 38, out_n)) out[out_n] = it;
          ++out_n;
        }
      }
      if (zdrop) {
        // the end gaps (tlen-end_h insertions, plen-end_v deletions) only
        // lower the score, so the maximal-score trim of the whole CIGAR ends
        // inside the walked part; a count past them leaves no CIGAR
        if (pops > (tlen - end_h) + (plen - end_v)) bad = true;
        if (!bad) {
          __syncwarp();
          if (lane == 0) {
            int len = out_n, sc = 0, ev = 0, eh = 0;
            fin_status = kStPartial;
            if (A2P && out_n == 0) {
              // an empty affine2p CIGAR is not trimmed (alignment/cigar_utils.c:
              // 281); gaps alone trim to nothing
              const bool gaps = (tlen - end_h) + (plen - end_v) > pops;
              fin_score = gaps ? INT32_MIN : s;
              fin_v = fin_h = -1;
            } else {
              if (lin) maxtrim_linear(p, out, &len, &sc, &ev, &eh);
              else maxtrim<A2P>(p, out, &len, &sc, &ev, &eh);
              fin_score = sc;
              fin_v = ev;
              fin_h = eh;
              out_n = len;
            }
          }
        }
      } else if (v != end_v || h != end_h) {
        bad = true;
      }
      if (EF && !bad && !zdrop) {
        // the free end: insertions, then deletions, up to the sequences' ends
        // (wavefront/wavefront_backtrace.c:346-356)
        const int ni = tlen - end_h, nd = plen - end_v;
        for (int j = lane; j < ni + nd; j += 32)
          if (CHK(out_n + j < plen + tlen, 40, out_n + j)) out[out_n + j] = j < ni ? 'I' : 'D';
        out_n += ni + nd;
        if (p.extension) {
          __syncwarp();
          if (lane == 0) {
            int len = out_n, sc = 0, ev = 0, eh = 0;
            const bool trimmed = lin ? maxtrim_linear(p, out, &len, &sc, &ev, &eh)
                                     : maxtrim<A2P>(p, out, &len, &sc, &ev, &eh);
            if (edit_like || (A2P && out_n == 0)) {
              // edit and indel are not trimmed (wavefront/wavefront_aligner.c:
              // 664-676), nor is an empty affine2p CIGAR (alignment/cigar_utils.c:
              // 281): the CIGAR stays as the back-trace wrote it, with the WFA
              // score and no end position
              fin_score = s;
              fin_v = fin_h = -1;
            } else {
              fin_status = trimmed ? kStPartial : kStCompleted;
              fin_score = sc;
              fin_v = ev;
              fin_h = eh;
              out_n = len;
            }
          }
        }
      }
    }
    if (t == 0) {
      p.status[pair] = bad ? kStUnattainable : fin_status;
      p.scores[pair] = bad ? (zdrop ? 0 : score) : fin_score;
      p.ops_len[pair] = bad ? 0 : out_n;
      if (p.end_info) {
        p.end_info[3 * (int64_t)pair] = bad ? -1 : fin_v;
        p.end_info[3 * (int64_t)pair + 1] = bad ? -1 : fin_h;
        p.end_info[3 * (int64_t)pair + 2] = s;
      }
    }
    group_sync<G>();
  }
}

}  // namespace wf2g

namespace wf2g {

// Kernel table of one family (wf-adaptive H, group size G, ends-free EF):
// (affine2p?, full CIGAR?, 2- or 8-bit staging, 2- or 4-byte offsets,
// single-component metric?) -> the kernel.  Taking the addresses instantiates
// the family in the including unit; CTA-per-pair families exist for
// full-CIGAR runs only (nullptr else).
template <typename T, bool H, int G, bool EF, bool L>
void* align_kernel_tl(int a2p, int cigar, int enc) {
  if (cigar) {
    if (enc == 2) return a2p && !L ? (void*)wfa_align_kernel<!L, true, 2, T, H, G, EF, L>
                                   : (void*)wfa_align_kernel<false, true, 2, T, H, G, EF, L>;
    return a2p && !L ? (void*)wfa_align_kernel<!L, true, 8, T, H, G, EF, L>
                     : (void*)wfa_align_kernel<false, true, 8, T, H, G, EF, L>;
  }
  if constexpr (G == 32) {
    if (enc == 2) return a2p && !L ? (void*)wfa_align_kernel<!L, false, 2, T, H, G, EF, L>
                                   : (void*)wfa_align_kernel<false, false, 2, T, H, G, EF, L>;
    return a2p && !L ? (void*)wfa_align_kernel<!L, false, 8, T, H, G, EF, L>
                     : (void*)wfa_align_kernel<false, false, 8, T, H, G, EF, L>;
  }
  return nullptr;
}
template <bool H, int G, bool EF>
void* align_kernel(int a2p, int cigar, int enc, int off_bytes, int lin) {
  if (lin) return off_bytes == 2 ? align_kernel_tl<int16_t, H, G, EF, true>(0, cigar, enc)
                                 : align_kernel_tl<int32_t, H, G, EF, true>(0, cigar, enc);
  return off_bytes == 2 ? align_kernel_tl<int16_t, H, G, EF, false>(a2p, cigar, enc)
                        : align_kernel_tl<int32_t, H, G, EF, false>(a2p, cigar, enc);
}

}  // namespace wf2g

// wfa_bialign.cuh -- device-side structures of the BiWFA (ultralow memory)
// path: the breakpoint search of wavefront/wavefront_bialign.c:975-1083 run as
// one CTA per segment, the sequence packing it reads, and the CIGAR gather
// that stitches the base-case pieces together.
//
// A segment is one call of wavefront_bialign_alignment
// (wavefront/wavefront_bialign.c:1145-1222): a pattern range [pb,pe) and a
// text range [tb,te) of one pair, entered in component cb and left in
// component ce.  Components: 0 M, 1 I1, 2 D1, 3 I2, 4 D2.
#pragma once
#include <cstdint>

#include "wfa_kernels.cuh"

namespace wf2g {

enum : int { kCompM = 0, kCompI1 = 1, kCompD1 = 2, kCompI2 = 3, kCompD2 = 4 };

// Breakpoint-search outcome (BiOut::status).
enum : int {
  kBiOk = 0,           // breakpoint found
  kBiEndReached = 1,   // one direction reached its end first (score in `reached`)
  kBiUnreachable = 2,  // more than max_score_scope NULL wavefronts in a row
  kBiMaxSteps = 3,     // score_forward + score_reverse reached max_steps
  kBiGuard = 4         // above the score bound of the segment: never expected
};

struct BiSeg {
  int32_t pair, pb, pe, tb, te, cb, ce, pad;
};

// wf_bialign_breakpoint_t (wavefront/wavefront_bialign.h) plus the status.
struct BiOut {
  int32_t status, reached, score, score_f, score_r, k_f, off_f, comp;
};

struct BiParams {
  Penalties pen;  // x, o1, e1, o2, e2 as in the unidirectional kernel
  // distance metric: 0 indel, 1 edit, 2 gap-linear (one component: the
  // gap-affine recurrence with e1 = 0 and no I/D inputs), 3 gap-affine,
  // 4 gap-affine-2p
  int metric;
  int scope;      // max_score_scope: ring depth of every component
  int max_steps;
  // heuristic of the forward/reverse searches (strategy bits, 0: none; no
  // z-drop) and its parameters
  int heur, h_min_len, h_max_dist, h_steps;
  int h_xdrop, h_min_k, h_max_k;
  // sequences: caller bytes, and the 2-bit packed copy of ACGT-only pairs
  const uint8_t* seqs;
  const int64_t* p_off;
  const int64_t* t_off;
  const uint32_t* packed;
  const int64_t* pk_p;  // word offset of pattern / text of a pair in `packed`
  const int64_t* pk_t;
  const uint8_t* enc2;  // 1: the pair is ACGT-only and packed
  // work
  const BiSeg* segs;
  int nseg;
  int32_t* queue;  // zeroed before launch
  BiOut* out;
  // per-CTA wavefront rows: 2 directions x components x scope slots + a NULL
  // row, `stride` int32 each, diagonal k at element k + kofs
  int32_t* rows;
  int64_t rows_per_cta;
  int stride;
  int kofs;
};

struct PackParams {
  const uint8_t* seqs;
  const int64_t* p_off;
  const int32_t* p_len;
  const int64_t* t_off;
  const int32_t* t_len;
  uint32_t* packed;
  const int64_t* pk_p;
  const int64_t* pk_t;
  uint8_t* enc2;
  int n;
};

// Words of one packed sequence: one padding word before, two after.
__host__ __device__ inline int64_t packed_words(int len) { return (int64_t)((len + 15) >> 4) + 3; }

// One piece of an output CIGAR: `len` bytes from src (fill == 0) or `len`
// copies of fill ('D' / 'I').
struct CopyDesc {
  int64_t src, dst;
  int32_t len, fill;
};

}  // namespace wf2g

// wfa_kernels.cuh -- device-side data structures of the GB300 wavefront aligner.
//
// One warp aligns one pair at a time (lanes striped over diagonals k),
// pulling pair indices from a device work queue.  Per warp:
//   shared memory  both sequences, packed 2 bits per base (16 bases per 32-bit
//                  word, first base in the most significant bits) or 1 byte per
//                  base (8 per 64-bit word) for non-ACGT input; the per-row
//                  limits of the wavefront ring;
//   global memory  (a private slice, L1/L2 resident) the wavefront ring: the
//                  last max_score_scope M rows and the last e+1 I/D rows, each
//                  row indexed by k + kofs over every diagonal the pair can
//                  reach, plus one all-NULL row; and, for full-CIGAR runs, one
//                  back-trace choice byte per computed cell.
#pragma once
#include <cstdint>

namespace wf2g {

// Offsets: any negative value is NULL; stored NULLs are canonical.
constexpr int32_t kNull = INT32_MIN / 2;  // wavefront/wavefront_offset.h:46
constexpr unsigned kFull = 0xffffffffu;

// Per-pair status values written by the kernels (wavefront/wfa.h:46-55).
constexpr int kStCompleted = 0;
constexpr int kStPartial = 1;
constexpr int kStMaxSteps = -100;
constexpr int kStOOM = -200;
constexpr int kStUnattainable = -300;
// no reference counterpart: ends-free lengths longer than the pair's
// sequences (the reference prints an error and exits,
// wavefront/wavefront_align.c:90-101)
constexpr int kStInvalidForm = -400;

// Back-trace choice byte, one per computed cell (s,k):
//   bits 0-2  source of M:  0 mismatch, 1 D1, 2 I1, 3 D2, 4 I2
//   bit 3     I1 extends (else opens)    bit 4  D1 extends
//   bit 5     I2 extends                 bit 6  D2 extends
enum : uint8_t { kSrcX = 0, kSrcD1 = 1, kSrcI1 = 2, kSrcD2 = 3, kSrcI2 = 4 };
// choice byte of an ends-free begin cell entered after score 0 (match < 0)
constexpr uint8_t kBegin = 0x80;

// Back-trace row table entry, one per score: choice bytes of the row's cells
// [lo, lo+width) start at byte `pos` of the back-trace store (the warp's slice,
// or the block pool); width < 0 marks a score without wavefront.
struct BtRow {
  int64_t pos;
  int32_t lo, width;
};
constexpr int kBtRowBytes = (int)sizeof(BtRow);

// Shared memory a CTA-per-pair group adds for its cross-warp reductions.
constexpr int kGroupRedBytes = 1024;

struct Penalties {
  int match;  // user match (<= 0)
  int x, o1, e1, o2, e2;  // internal (possibly Eizenga-transformed) penalties
  int R;    // M ring depth = max_score_scope
  int RI1;  // I1/D1 ring depth = e1+1
  int RI2;  // I2/D2 ring depth = e2+1 (affine2p)
};

// heuristic strategy bits (wavefront/wavefront_heuristic.h:41-49)
constexpr int kHsBandedStatic = 0x01, kHsBandedAdaptive = 0x02, kHsWfadaptive = 0x04;
constexpr int kHsXdrop = 0x10, kHsZdrop = 0x20, kHsWfmash = 0x40;

struct KParams {
  Penalties pen;
  // distance metric (wavefront/wavefront_penalties.h:42-48): 0 indel, 1 edit,
  // 2 gap-linear -- one component, run on the gap-affine recurrence with e1 = 0
  // and no I/D inputs, which is the same recurrence -- 3 gap-affine, 4
  // gap-affine-2p
  int metric;
  int max_steps;
  // heuristic strategy bits (wavefront/wavefront_heuristic.h:41-49; 0: none)
  // and parameters: min wavefront length, max distance threshold, steps
  // between cut-offs, x-drop, z-drop, band limits (:51-69)
  int heur, h_min_len, h_max_dist, h_steps;
  int h_xdrop, h_zdrop, h_min_k, h_max_k;
  // inputs
  const uint8_t* seqs;
  const int64_t* p_off;
  const int32_t* p_len;
  const int64_t* t_off;
  const int32_t* t_len;
  // components the alignment of a pair begins and ends in (0 M, 1 I1, 2 D1,
  // 3 I2, 4 D2; nullptr: M), for the BiWFA base cases
  const int8_t* comp_begin;
  const int8_t* comp_end;
  // work list: items[i] is a pair index (items == nullptr: identity)
  const int32_t* items;
  const int32_t* num_items_dev;  // if non-null, overrides n_items
  int n_items;
  int32_t* queue;  // work-queue head (zeroed before launch)
  // retry list for pairs this pass cannot finish (non-ACGT / back-trace overflow)
  int32_t* retry_items;
  int32_t* retry_count;
  int final_pass;  // 1: report overflow as WF_STATUS_OOM instead of retrying
  // outputs
  int32_t* scores;
  int32_t* status;
  uint8_t* ops;
  const int64_t* ops_off;
  int32_t* ops_len;
  // geometry of this pass
  int max_len;        // longest sequence of the batch
  int row_stride;     // ring row length (elements), >= 2*max_len+6
  int kofs;           // diagonal k lives at element k+kofs of a row
  int seq_in_smem;    // 1: staged sequences in shared memory, 0: in gscratch
  int smem_per_group;  // bytes
  uint8_t* gscratch;  // per-warp global slices
  int64_t gscratch_per_group;
  // per-warp slice: [ring: (nrows+1) rows][sequences if !seq_in_smem][table][bits]
  int64_t ring_bytes;
  int64_t seq_bytes;
  int table_cap;      // back-trace row table entries (scores); also the score bound
  int64_t bits_cap;   // back-trace choice bytes per warp (pooled: owned-block list + walk items)
  // Back-trace block pool (nullptr: choice bytes in the warp's slice).  A pair
  // takes blocks from a shared free stack as its rows need room and returns
  // them when it finishes, so each pair uses what its alignment needs.
  uint8_t* pool;
  int64_t block_bytes;  // >= the widest row
  int32_t* pool_stack;  // free block indices
  int32_t* pool_count;  // entries on the stack
  int32_t* pool_lock;   // 0 free, 1 held
  int max_blocks;       // blocks one pair may hold
  int64_t pair_cap;     // choice bytes one pair may use (its back-trace budget)
  // a pass with a retry list sends pairs this long or longer (either
  // sequence) straight to it: the CTA-per-pair passes take them (0: off)
  int wide_min_len;
  // ends-free form (kernels built with EF; wavefront/wavefront_attributes.h:
  // 55-69): free lengths, or the extension presets per pair
  // (wavefront/wavefront_align.c:57-63) followed by maximal-score trimming
  // with the user's penalties um..ue2 (alignment/cigar_utils.c:112-318)
  int pbf, pef, tbf, tef, extension;
  int um, ux, uo1, ue1, uo2, ue2;
  // optional per-pair {cigar->end_v, cigar->end_h, WFA score} (nullptr: none)
  int32_t* end_info;
};

// int16 NULL of the shared-memory rows (offsets stay below 32,000)
constexpr int kNull16 = -32768;

// Launch parameters of the shared-memory fast pass (wfa_fast.cu), filled by
// the engine (wfa_engine.cu).
struct FastParams {
  int x, oe, e;   // penalties divided by g: mismatch, gap open+extend, gap extend
  int g;          // gcd(x, o+e, e)
  int match;      // the user's match (<= 0), for the classic score
  int R, RI;      // ring depths: max(x, oe) + 1 M rows, e + 1 I and D rows
  int max_steps;  // unscaled step limit (INT32_MAX: none)
  // wf-adaptive cut-off (two-diagonal kernel): min_wavefront_length,
  // max_distance_threshold, steps_between_cutoffs
  int h_min_len, h_max_dist, h_steps;
  // first pass: the projected final scaled score beyond which a pair leaves
  // for the wider rows at the probe step
  int probe_limit;
  // the diagonals a pass computes, [-reach, reach]: its rows' W/2 - 4, or
  // fewer in the first pass to send pairs to the wider ones
  int reach;
  const uint8_t* seqs;
  const int64_t* p_off;
  const int32_t* p_len;
  const int64_t* t_off;
  const int32_t* t_len;
  // work list: items[i] is a pair index (items == nullptr: identity, n_items
  // pairs); num_items_dev, if non-null, holds the list's length
  const int32_t* items;
  const int32_t* num_items_dev;
  int n_items;
  int32_t* queue;        // work-queue head (zeroed before launch)
  int32_t* retry_items;  // pairs left to the next pass
  int32_t* retry_count;
  int32_t* scores;
  int32_t* status;
  uint8_t* ops;
  const int64_t* ops_off;
  int32_t* ops_len;
  int32_t* end_info;  // optional {end_v, end_h, WFA score} per pair
  int max_len;        // longest sequence of the batch (a longer pair is punted)
  int nq;             // 64-bit word pairs staged per sequence
  int rows_off, q_off, meta_off, red_off;  // byte offsets of the parts of a group's shared memory
  uint8_t* scratch;     // per-group global slices
  int64_t slice_bytes;  // [choice codes: s_cap rows][row limits: s_cap][walk items]
  int s_cap;            // scaled scores a slice holds
  int64_t pair_cap;     // back-trace bytes one pair may use (0: no cap); a pair
                        // over it is left to the general kernel, which reports
                        // WF_STATUS_OOM for it
  int64_t items_off;
  int64_t items_cap;
};

}  // namespace wf2g

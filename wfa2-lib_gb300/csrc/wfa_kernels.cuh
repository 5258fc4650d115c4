// wfa_kernels.cuh -- device-side data structures of the GB300 wavefront aligner.
//
// One warp aligns one pair at a time (lane = a stripe of diagonals), pulling
// pair indices from a device work queue.  Per warp the kernel keeps, in shared
// memory (or, for wide wavefronts, in a private slice of global memory):
//   * both sequences, packed 2 bits per base (32 bases per 64-bit word, first
//     base in the most significant bits) or 8 bits per byte for non-ACGT input;
//   * a ring of the last max_score_scope M-wavefronts and the last e+1 I/D
//     wavefronts, indexed by (k mod WCAP);
//   * the ring's per-row limits.
// Full-CIGAR runs also write, per computed cell, one byte of back-trace choice
// bits into a per-warp global region; the device back-trace walks those bytes.
#pragma once
#include <cstdint>

namespace wf2g {

// Offsets are int32; any negative value is NULL.  Stored NULLs are canonical.
constexpr int32_t kNull = INT32_MIN / 2;  // wavefront/wavefront_offset.h:46
constexpr unsigned kFull = 0xffffffffu;

// Per-pair status values written by the kernels (reference codes, wavefront/wfa.h:46-55,
// plus internal retry codes that never reach the caller).
constexpr int kStCompleted = 0;
constexpr int kStPartial = 1;
constexpr int kStMaxSteps = -100;
constexpr int kStOOM = -200;
constexpr int kStUnattainable = -300;
constexpr int kStRetry = -1000;  // internal: re-run in the next pass

// Back-trace choice byte, one per computed cell (s,k):
//   bits 0-2  source of M:  0 mismatch, 1 D1, 2 I1, 3 D2, 4 I2
//   bit 3     I1 extends (else opens)    bit 4  D1 extends
//   bit 5     I2 extends                 bit 6  D2 extends
enum : uint8_t { kSrcX = 0, kSrcD1 = 1, kSrcI1 = 2, kSrcD2 = 3, kSrcI2 = 4 };

struct Penalties {
  int match;  // <= 0 (transformed set keeps the original match)
  int x, o1, e1, o2, e2;
  int R;    // M ring depth = max_score_scope
  int RI1;  // I1/D1 ring depth = e1+1
  int RI2;  // I2/D2 ring depth = e2+1 (affine2p)
};

struct KParams {
  Penalties pen;
  int max_steps;
  // inputs
  const uint8_t* seqs;
  const int64_t* p_off;
  const int32_t* p_len;
  const int64_t* t_off;
  const int32_t* t_len;
  // work list: items[i] is a pair index (items == nullptr: identity)
  const int32_t* items;
  const int32_t* num_items_dev;  // if non-null, overrides n_items
  int n_items;
  int32_t* queue;  // work-queue head (zeroed before launch)
  // retry list for pairs this pass cannot finish (overflow / non-ACGT)
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
  int wcap;          // ring width, power of two
  int max_len;       // longest sequence staged by this pass
  int ring_in_smem;  // 1: ring in shared memory, 0: in gscratch
  int seq_in_smem;   // 1: staged sequences in shared memory, 0: in gscratch
  int smem_per_warp; // bytes
  uint8_t* gscratch; // per-warp global scratch
  int64_t gscratch_per_warp;
  // per-warp gscratch slice: [ring if !ring_in_smem][P,T if !seq_in_smem][table][bits]
  int64_t ring_bytes_global;
  int64_t seq_bytes_global;
  int table_cap;     // back-trace row table entries (scores)
  int64_t bits_cap;  // back-trace choice bytes per warp
};

// Host-side helpers shared with the engine.
struct Geometry {
  int nrows;            // ring rows
  int seq_words;        // 64-bit words per staged sequence
  int smem_per_warp;    // bytes of shared memory per warp
};

}  // namespace wf2g

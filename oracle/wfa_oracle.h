/*
 * wfa_oracle.h -- CPU restatement of WFA2-lib's exact wavefront alignment.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against (tests/, __graft_entry__.smoke(), and the cpu_baseline /
 * --impl reference legs of bench.py).  It is never linked into, loaded by or
 * called from the product library (wfa2-lib_gb300/).
 *
 * Parity is pinned: tests/test_oracle_golden.py checks this restatement against
 * every in-scope golden file of the reference test-suite
 * (tests/wfa.utest.check/*.alg, 305 pairs), and tests/golden/ holds outputs of
 * the reference itself (built from its sources by oracle/Makefile) on seeded
 * synthetic pairs.
 */
#ifndef WFA_ORACLE_H_
#define WFA_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Configuration vector (plain ints, ctypes friendly).
 *   cfg[0] distance metric   (3 = gap_affine, 4 = gap_affine_2p; wavefront/wavefront_penalties.h:42-48)
 *   cfg[1] match  (<= 0)     cfg[2] mismatch (> 0)
 *   cfg[3] gap_opening1      cfg[4] gap_extension1
 *   cfg[5] gap_opening2      cfg[6] gap_extension2   (affine2p only)
 *   cfg[7] memory mode       (0 high, 1 med, 2 low, 3 ultralow)
 *   cfg[8] score only        (1 = compute_score, 0 = compute_alignment)
 *   cfg[9] max alignment steps (<= 0 means unlimited)
 *   cfg[10] heuristic        (0 none, 1 wf-adaptive)
 *   cfg[11..13] wf-adaptive min_wavefront_length, max_distance_threshold,
 *           steps_between_cutoffs (wavefront/wavefront_heuristic.h:42-69)
 *   cfg[14] span             (0 end-to-end, 1 ends-free; wavefront/wavefront_attributes.h:55-69)
 *   cfg[15..18] pattern_begin_free, pattern_end_free, text_begin_free,
 *           text_end_free
 *   cfg[19] extension        (1: ends-free with the extension presets and
 *           maximal-score trimming, wavefront/wavefront_align.c:57-63)
 *   cfg[20] heuristic strategy bit set (wf_heuristic_strategy,
 *           wavefront/wavefront_heuristic.h:41-49); non-zero overrides cfg[10]
 *   cfg[21] xdrop  cfg[22] zdrop  cfg[23] band min_k  cfg[24] band max_k
 */
#define ORACLE_CFG_LEN 25

/* Align num_pairs pairs with nthreads host threads (OpenMP, one aligner per
 * thread, as tools/align_benchmark/align_benchmark.c:504-586 does).
 *   sequences       concatenated ASCII buffer
 *   p_off/p_len     pattern offsets/lengths into it, t_off/t_len likewise
 *   out_score       cigar->score as the reference reports it
 *   out_status      align_status.status (WF_STATUS_*)
 *   out_ops         CIGAR operations ('M','X','I','D'); pair i writes at
 *                   ops_off[i] and may use up to p_len[i]+t_len[i] bytes.
 *                   May be NULL in score-only mode.
 *   out_ops_len     number of operations written (0 in score-only mode)
 *   out_cells       optional (may be NULL): WFA cells computed for the pair
 *                   (sum over scores of hi-lo+1 of the compute loop)
 *   out_ext         optional (may be NULL): characters matched by extend
 *                   (sum of offset increments over all extended diagonals)
 *   out_end         optional (may be NULL): cigar->end_v, cigar->end_h of
 *                   pair i at out_end[2i], out_end[2i+1]
 * Returns 0, or -1 on an invalid configuration.  A pair whose ends-free
 * parameters exceed its lengths (the reference prints an error and exits,
 * wavefront/wavefront_align.c:90-101) gets status ORACLE_STATUS_INVALID_FORM. */
#define ORACLE_STATUS_INVALID_FORM (-400)
int oracle_align_batch(
    const int* cfg, int num_pairs,
    const char* sequences,
    const int64_t* p_off, const int32_t* p_len,
    const int64_t* t_off, const int32_t* t_len,
    int32_t* out_score, int32_t* out_status,
    char* out_ops, const int64_t* ops_off, int32_t* out_ops_len,
    int64_t* out_cells, int64_t* out_ext, int32_t* out_end, int nthreads);

/* The same, with out_flags[i] (may be NULL) receiving ORACLE_FLAG_* bits.  A
 * CIGAR longer than p_len[i]+t_len[i] is reported with out_ops_len[i] = -1. */
#define ORACLE_FLAG_STALE_SOURCE 1 /* back-trace read a wavefront a cut emptied */
#define ORACLE_FLAG_OVER_BOUND 2   /* ran past the reference's per-pair wavefront table */
int oracle_align_batch_flags(
    const int* cfg, int num_pairs,
    const char* sequences,
    const int64_t* p_off, const int32_t* p_len,
    const int64_t* t_off, const int32_t* t_len,
    int32_t* out_score, int32_t* out_status,
    char* out_ops, const int64_t* ops_off, int32_t* out_ops_len,
    int64_t* out_cells, int64_t* out_ext, int32_t* out_end, int32_t* out_flags, int nthreads);

/* Compares batch a (the results under test) with batch b (the checker's)
 * pair by pair, and replays and rescores every CIGAR of a whose status is 0
 * (wfa_check.c).  a_ops/b_ops may both be NULL (score-only).  out[0..5]:
 * score mismatches, status mismatches, CIGAR mismatches, CIGARs of a that do
 * not align their pair, CIGARs of a whose rescored score differs from a's
 * score, and the first differing pair (-1: none). */
int oracle_compare_batch(const int* cfg, int num_pairs, const char* sequences,
                         const int64_t* p_off, const int32_t* p_len,
                         const int64_t* t_off, const int32_t* t_len,
                         const int32_t* a_score, const int32_t* a_status, const char* a_ops,
                         const int64_t* a_ops_off, const int32_t* a_ops_len,
                         const int32_t* b_score, const int32_t* b_status, const char* b_ops,
                         const int64_t* b_ops_off, const int32_t* b_ops_len, int nthreads,
                         int64_t* out);

#ifdef __cplusplus
}
#endif
#endif /* WFA_ORACLE_H_ */

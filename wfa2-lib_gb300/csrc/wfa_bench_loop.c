/*
 * wfa_bench_loop.c -- benchmark helper: the plain per-pair drop-in usage.
 *
 * A C caller of WFA2-lib aligns a batch by calling wavefront_align() once per
 * pair (tools/align_benchmark/align_benchmark.c:452-503).  This loop does
 * exactly that against libwfa2gpu.so, so the per-pair GPU path is timed
 * without any interpreter overhead.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdint.h>
#include <time.h>

#include "wfa2gpu.h"

double wf2g_bench_per_pair(wavefront_aligner_t* wf, int n, const char* seqs,
                           const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                           const int32_t* t_len, int32_t* scores, int32_t* status,
                           int32_t* ops_len) {
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  for (int i = 0; i < n; ++i) {
    status[i] = wavefront_align(wf, seqs + p_off[i], p_len[i], seqs + t_off[i], t_len[i]);
    scores[i] = wf->cigar->score;
    ops_len[i] = wf->cigar->end_offset - wf->cigar->begin_offset;
  }
  clock_gettime(CLOCK_MONOTONIC, &b);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}

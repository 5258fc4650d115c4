/*
 * wfa_check.c -- pair-by-pair comparison of two batches of alignment results
 * (the GPU's and the CPU checker's), with a replay and a rescoring of every
 * CIGAR of the first batch.
 *
 * TEST INFRASTRUCTURE ONLY: called by tests/ and by bench.py's parity check of
 * the timed batch; never linked into or called by the product library.
 *
 * Replay restates cigar_check_alignment (alignment/cigar.c:347-417): every 'M'
 * must pair equal bytes, every 'X' different bytes, and the operations must
 * consume both sequences exactly.  Rescoring restates cigar_score_gap_affine
 * (alignment/cigar.c:277-303: a gap run pays gap_opening once) and
 * cigar_score_gap_affine2p (:304-346: each run pays the cheaper of its two
 * gap models), with the user's penalties (match <= 0).
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "wfa_oracle.h"

static int replay_ok(const char* P, int plen, const char* T, int tlen, const char* ops, int n) {
  int v = 0, h = 0;
  for (int i = 0; i < n; ++i) {
    switch (ops[i]) {
      case 'M':
        if (v >= plen || h >= tlen || P[v] != T[h]) return 0;
        ++v;
        ++h;
        break;
      case 'X':
        if (v >= plen || h >= tlen || P[v] == T[h]) return 0;
        ++v;
        ++h;
        break;
      case 'I':
        if (h >= tlen) return 0;
        ++h;
        break;
      case 'D':
        if (v >= plen) return 0;
        ++v;
        break;
      default:
        return 0;
    }
  }
  return v == plen && h == tlen;
}

static int run_cost_2p(const int* cfg, char op, int len) {
  switch (op) {
    case 'M': return cfg[1] * len;
    case 'X': return cfg[2] * len;
    default: {
      const int s1 = cfg[3] + cfg[4] * len, s2 = cfg[5] + cfg[6] * len;
      return s1 < s2 ? s1 : s2;
    }
  }
}

/* Score of a CIGAR under the configuration's penalties (cfg as in
 * wfa_oracle.h: [0] metric 3 gap-affine / 4 gap-affine-2p, [1] match,
 * [2] mismatch, [3..6] gap_opening1, gap_extension1, gap_opening2,
 * gap_extension2). */
static int rescore(const int* cfg, const char* ops, int n) {
  int score = 0;
  if (cfg[0] == 4) {
    char last = 0;
    int run = 0;
    for (int i = 0; i < n; ++i) {
      if (ops[i] != last && last != 0) {
        score -= run_cost_2p(cfg, last, run);
        run = 0;
      }
      last = ops[i];
      ++run;
    }
    if (last) score -= run_cost_2p(cfg, last, run);
    return score;
  }
  char last = 0;
  for (int i = 0; i < n; ++i) {
    switch (ops[i]) {
      case 'M': score -= cfg[1]; break;
      case 'X': score -= cfg[2]; break;
      case 'D': score -= cfg[4] + (last == 'D' ? 0 : cfg[3]); break;
      case 'I': score -= cfg[4] + (last == 'I' ? 0 : cfg[3]); break;
      default: break;
    }
    last = ops[i];
  }
  return score;
}

int oracle_compare_batch(const int* cfg, int num_pairs, const char* seqs, const int64_t* p_off,
                         const int32_t* p_len, const int64_t* t_off, const int32_t* t_len,
                         const int32_t* a_score, const int32_t* a_status, const char* a_ops,
                         const int64_t* a_ops_off, const int32_t* a_ops_len,
                         const int32_t* b_score, const int32_t* b_status, const char* b_ops,
                         const int64_t* b_ops_off, const int32_t* b_ops_len, int nthreads,
                         int64_t* out) {
  int64_t sc = 0, st = 0, cg = 0, inv = 0, rs = 0;
  int64_t first = INT64_MAX;
  const int full = (a_ops != NULL && b_ops != NULL);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static, 1024) \
    reduction(+ : sc, st, cg, inv, rs) reduction(min : first)
#endif
  for (int i = 0; i < num_pairs; ++i) {
    int bad = 0;
    if (a_score[i] != b_score[i]) { ++sc; bad = 1; }
    if (a_status[i] != b_status[i]) { ++st; bad = 1; }
    if (full) {
      const int na = a_ops_len[i], nb = b_ops_len[i];
      const char* oa = a_ops + a_ops_off[i];
      if (na != nb || (na > 0 && memcmp(oa, b_ops + b_ops_off[i], (size_t)na) != 0)) {
        ++cg;
        bad = 1;
      }
      if (a_status[i] == 0) {
        if (!replay_ok(seqs + p_off[i], p_len[i], seqs + t_off[i], t_len[i], oa, na)) {
          ++inv;
          bad = 1;
        } else if (rescore(cfg, oa, na) != a_score[i]) {
          ++rs;
          bad = 1;
        }
      }
    }
    if (bad && i < first) first = i;
  }
  out[0] = sc;
  out[1] = st;
  out[2] = cg;
  out[3] = inv;
  out[4] = rs;
  out[5] = first == INT64_MAX ? -1 : first;
  return 0;
}

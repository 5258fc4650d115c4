/*
 * wfa_oracle_bialign.c -- CPU restatement of WFA2-lib's BiWFA (ultralow
 * memory mode).  TEST INFRASTRUCTURE ONLY (see wfa_oracle.h).
 *
 * Restates wavefront/wavefront_bialign.c:
 *   breakpoint checks        m2m :798-874, indel2indel :477-573
 *   overlap scan             :878-956 (D2,I2,D1,I1 then M per score; the lowest
 *                            k of a compare wins; a later candidate replaces
 *                            the breakpoint only with a strictly lower score)
 *   gap-open adjustment      :960-973
 *   breakpoint search        :975-1083 (forward/reverse alternate until their
 *                            max antidiagonals meet, then overlap-scan)
 *   end-reached exception    :1084-1114 (base case if score <= 500)
 *   recursion                :1145-1222 (trivial cases, base case if the
 *                            remaining score <= 250, halves split at the
 *                            breakpoint with its component as boundary)
 *   score-only               :1226-1263
 *   dispatcher               :1267-1294 (max length <= 100 -> base case)
 * The forward and reverse aligners are score-only (modular rows); the base
 * aligner keeps every wavefront (wavefront/wavefront_bialigner.c:40-74).
 */
#include <limits.h>
#include <stdlib.h>
#include <string.h>

#include "wfa_oracle_internal.h"

#define BI_FALLBACK_MIN_SCORE 250
#define BI_FALLBACK_MIN_LENGTH 100
#define BI_RECOVERY_MIN_SCORE 500
#define ST_OK (-1)

typedef struct {
  int score, score_f, score_r, k_f, k_r, off_f, off_r, comp;
} bp_t;

typedef struct {
  const pen_t* p;
  const char *P, *T, *Prev, *Trev;
  int plen, tlen;
  oracle_ws_t wsf, wsr, wsb;
  oracle_ua_t F, R;
  char* ops;
  int nops;
  int score; /* cigar->score */
  int split0; /* the top level split at a breakpoint (it alone sets the CIGAR's end) */
  int64_t cells, ext; /* work counters: wavefront cells computed, bases matched */
} bi_t;

/* wavefront/wavefront_bialign.c:798-874 */
static void bp_m2m(int plen, int tlen, int forward, int score_0, int score_1, const orow_t* w0,
                   const orow_t* w1, bp_t* bp) {
  if (score_0 + score_1 >= bp->score) return;
  const int lo_0 = w0->lo, hi_0 = w0->hi;
  const int lo_1 = tlen - plen - w1->hi, hi_1 = tlen - plen - w1->lo;
  if (hi_1 < lo_0 || hi_0 < lo_1) return;
  const int min_hi = hi_0 < hi_1 ? hi_0 : hi_1;
  const int max_lo = lo_0 > lo_1 ? lo_0 : lo_1;
  for (int k0 = max_lo; k0 <= min_hi; ++k0) {
    const int k1 = tlen - plen - k0;
    const int32_t o0 = w0->off[k0], o1 = w1->off[k1];
    if (o0 + o1 >= tlen) {
      if (forward) {
        bp->score_f = score_0; bp->score_r = score_1;
        bp->k_f = k0; bp->k_r = k1; bp->off_f = o0; bp->off_r = o1;
      } else {
        bp->score_f = score_1; bp->score_r = score_0;
        bp->k_f = k1; bp->k_r = k0; bp->off_f = o1; bp->off_r = o0;
      }
      bp->score = score_0 + score_1;
      bp->comp = C_M;
      return;
    }
  }
}

/* wavefront/wavefront_bialign.c:477-573 */
static void bp_indel(int plen, int tlen, int forward, int score_0, int score_1, const orow_t* w0,
                     const orow_t* w1, int comp, int gap_open, bp_t* bp) {
  const int lo_0 = w0->lo, hi_0 = w0->hi;
  const int lo_1 = tlen - plen - w1->hi, hi_1 = tlen - plen - w1->lo;
  if (hi_1 < lo_0 || hi_0 < lo_1) return;
  const int min_hi = hi_0 < hi_1 ? hi_0 : hi_1;
  const int max_lo = lo_0 > lo_1 ? lo_0 : lo_1;
  if (score_0 + score_1 - gap_open >= bp->score) return;
  for (int k0 = max_lo; k0 <= min_hi; ++k0) {
    const int k1 = tlen - plen - k0;
    const int32_t o0 = w0->off[k0], o1 = w1->off[k1];
    if (o0 + o1 >= tlen) {
      if (forward) {
        if (o0 - k0 > plen || o0 > tlen) continue;
        bp->score_f = score_0; bp->score_r = score_1;
        bp->k_f = k0; bp->k_r = k1; bp->off_f = o0; bp->off_r = o1;
      } else {
        if (o1 - k1 > plen || o1 > tlen) continue;
        bp->score_f = score_1; bp->score_r = score_0;
        bp->k_f = k1; bp->k_r = k0; bp->off_f = o1; bp->off_r = o0;
      }
      bp->score = score_0 + score_1 - gap_open;
      bp->comp = comp;
      return;
    }
  }
}

static const orow_t* row_or_null(oracle_ws_t* ws, int s, int c) {
  const orow_t* r = oracle_row(ws, s, c);
  return r->exists ? r : NULL;
}

/* wavefront/wavefront_bialign.c:878-956 */
static void bp_overlap(const pen_t* p, oracle_ua_t* a0, oracle_ua_t* a1, int forward, bp_t* bp) {
  const int score_0 = a0->s, score_1 = a1->s;
  const int plen = a0->plen, tlen = a0->tlen;
  const orow_t* m0 = row_or_null(a0->ws, score_0, C_M);
  if (!m0) return;
  const orow_t* d1_0 = row_or_null(a0->ws, score_0, C_D1);
  const orow_t* i1_0 = row_or_null(a0->ws, score_0, C_I1);
  const orow_t* d2_0 = p->metric == 4 ? row_or_null(a0->ws, score_0, C_D2) : NULL;
  const orow_t* i2_0 = p->metric == 4 ? row_or_null(a0->ws, score_0, C_I2) : NULL;
  for (int i = 0; i < p->scope; ++i) {
    const int si = score_1 - i;
    if (si < 0) break;
    if (p->metric == 4) {
      if (score_0 + si - p->o2 >= bp->score) continue;
      const orow_t* d2_1 = row_or_null(a1->ws, si, C_D2);
      if (d2_0 && d2_1) bp_indel(plen, tlen, forward, score_0, si, d2_0, d2_1, C_D2, p->o2, bp);
      const orow_t* i2_1 = row_or_null(a1->ws, si, C_I2);
      if (i2_0 && i2_1) bp_indel(plen, tlen, forward, score_0, si, i2_0, i2_1, C_I2, p->o2, bp);
    }
    if (p->metric >= 3 && score_0 + si - p->o1 >= bp->score) continue;
    const orow_t* d1_1 = row_or_null(a1->ws, si, C_D1);
    if (d1_0 && d1_1) bp_indel(plen, tlen, forward, score_0, si, d1_0, d1_1, C_D1, p->o1, bp);
    const orow_t* i1_1 = row_or_null(a1->ws, si, C_I1);
    if (i1_0 && i1_1) bp_indel(plen, tlen, forward, score_0, si, i1_0, i1_1, C_I1, p->o1, bp);
    if (score_0 + si >= bp->score) continue;
    const orow_t* m1 = row_or_null(a1->ws, si, C_M);
    if (m1) bp_m2m(plen, tlen, forward, score_0, si, m0, m1, bp);
  }
}

/* wavefront/wavefront_bialign.c:975-1083.  Returns ST_OK, a stepper status
 * (ST_END_REACHED / ST_END_UNREACHABLE) or ST_MAX_STEPS; *reached_score gets
 * the score of the aligner that reached its end. */
static int find_breakpoint_(bi_t* b, int pb, int pe, int tb, int te, int cb, int ce, bp_t* bp,
                            int* reached_score) {
  const pen_t* p = b->p;
  const int plen = pe - pb, tlen = te - tb;
  oracle_ua_t* F = &b->F;
  oracle_ua_t* R = &b->R;
  oracle_ua_start(F, &b->wsf, p, b->P + pb, plen, b->T + tb, tlen, cb, ce);
  oracle_ua_start(R, &b->wsr, p, b->Prev + (b->plen - pe), plen, b->Trev + (b->tlen - te), tlen,
                  ce, cb);
  const int max_antidiagonal = plen + tlen - 1;
  int fmax = 0, rmax = 0, mak = 0, st;
  bp->score = INT_MAX;
  if ((st = oracle_ua_extend(F, &fmax))) { *reached_score = F->s; return st; }
  if ((st = oracle_ua_extend(R, &rmax))) { *reached_score = R->s; return st; }
  int last_forward = 0;
  while (1) {
    if (fmax + rmax >= max_antidiagonal) break;
    oracle_ua_compute(F);
    st = oracle_ua_extend(F, &mak);
    if (fmax < mak) fmax = mak;
    last_forward = 1;
    if (st) { *reached_score = F->s; return st; }
    if (fmax + rmax >= max_antidiagonal) break;
    oracle_ua_compute(R);
    st = oracle_ua_extend(R, &mak);
    if (rmax < mak) rmax = mak;
    last_forward = 0;
    if (st) { *reached_score = R->s; return st; }
    if (R->s + F->s >= p->max_steps) return ST_MAX_STEPS;
  }
  /* wavefront/wavefront_bialign.c:960-973 (0 for the single-component metrics) */
  const int gap_opening = p->metric == 4 ? (p->o1 > p->o2 ? p->o1 : p->o2) : p->metric == 3 ? p->o1 : 0;
  const int scope = p->scope;
  while (1) {
    if (last_forward) {
      const int min_sr = R->s > scope - 1 ? R->s - (scope - 1) : 0;
      if (F->s + min_sr - gap_opening >= bp->score) break;
      bp_overlap(p, F, R, 1, bp);
      oracle_ua_compute(R);
      if ((st = oracle_ua_extend(R, NULL))) { *reached_score = R->s; return st; }
    }
    const int min_sf = F->s > scope - 1 ? F->s - (scope - 1) : 0;
    if (min_sf + R->s - gap_opening >= bp->score) break;
    bp_overlap(p, R, F, 0, bp);
    oracle_ua_compute(F);
    if ((st = oracle_ua_extend(F, NULL))) { *reached_score = F->s; return st; }
    if (R->s + F->s >= p->max_steps) return ST_MAX_STEPS;
    last_forward = 1;
  }
  return ST_OK;
}

static int find_breakpoint(bi_t* b, int pb, int pe, int tb, int te, int cb, int ce, bp_t* bp,
                           int* reached_score) {
  const int st = find_breakpoint_(b, pb, pe, tb, te, cb, ce, bp, reached_score);
  b->cells += b->F.cells + b->R.cells;
  b->ext += b->F.ext + b->R.ext;
  return st;
}

/* wavefront/wavefront_bialign.c:159-194: regular WFA on the sub-problem with
 * the given boundary components, appended to the CIGAR. */
static int bi_base(bi_t* b, int pb, int pe, int tb, int te, int cb, int ce) {
  const pen_t* p = b->p;
  oracle_ua_t U;
  oracle_ua_start(&U, &b->wsb, p, b->P + pb, pe - pb, b->T + tb, te - tb, cb, ce);
  U.heur = 0; /* the base aligner's heuristic is none (wavefront/wavefront_bialigner.c:64-66) */
  int st;
  while (1) {
    st = oracle_ua_extend(&U, NULL);
    if (st) break;
    oracle_ua_compute(&U);
    b->cells += U.cells;
    U.cells = 0;
    if (U.s >= p->max_steps) {
      /* wavefront/wavefront_unialign.c:102-107 sets the base CIGAR's score,
       * which wavefront_bialign_base copies before failing */
      b->score = -p->max_steps;
      return ST_UNATTAINABLE;
    }
  }
  b->ext += U.ext;
  if (st != ST_END_REACHED) return ST_UNATTAINABLE;
  const int n = oracle_ua_backtrace(&U, b->ops + b->nops);
  if (n < 0) return ST_UNATTAINABLE;
  b->nops += n;
  b->score = oracle_classic_score(p, pe - pb, te - tb, U.s);
  return ST_OK;
}

/* wavefront/wavefront_bialign.c:1145-1222 */
static int bi_alignment(bi_t* b, int pb, int pe, int tb, int te, int cb, int ce,
                        int score_remaining, int level) {
  const int plen = pe - pb, tlen = te - tb;
  if (tlen == 0) {
    for (int i = 0; i < plen; ++i) b->ops[b->nops++] = 'D';
    return ST_OK;
  }
  if (plen == 0) {
    for (int i = 0; i < tlen; ++i) b->ops[b->nops++] = 'I';
    return ST_OK;
  }
  if (score_remaining <= BI_FALLBACK_MIN_SCORE) return bi_base(b, pb, pe, tb, te, cb, ce);
  bp_t bp;
  int reached = 0;
  int st = find_breakpoint(b, pb, pe, tb, te, cb, ce, &bp, &reached);
  if (st != ST_OK) {
    /* wavefront/wavefront_bialign.c:1084-1114 */
    if (st == ST_END_REACHED) {
      if (reached <= BI_RECOVERY_MIN_SCORE) return bi_base(b, pb, pe, tb, te, cb, ce);
      return ST_END_UNREACHABLE;
    }
    return st;
  }
  const int bh = bp.off_f, bv = bp.off_f - bp.k_f;
  st = bi_alignment(b, pb, pb + bv, tb, tb + bh, cb, bp.comp, bp.score_f, level + 1);
  if (st != ST_OK) return st;
  st = bi_alignment(b, pb + bv, pe, tb + bh, te, bp.comp, ce, bp.score_r, level + 1);
  if (st != ST_OK) return st;
  if (level == 0) {
    b->score = oracle_classic_score(b->p, plen, tlen, bp.score);
    b->split0 = 1;
  }
  return ST_OK;
}

static char* reversed(const char* s, int n) {
  char* r = (char*)malloc((size_t)n + 1);
  for (int i = 0; i < n; ++i) r[i] = s[n - 1 - i];
  return r;
}

void oracle_bialign(const pen_t* p, const char* P, int plen, const char* T, int tlen,
                    oracle_ws_t* ws, int32_t* out_score, int32_t* out_status, char* ops,
                    int32_t* ops_len, int64_t* cells, int64_t* ext, int32_t* end) {
  (void)ws;
  bi_t b;
  memset(&b, 0, sizeof(b));
  b.p = p;
  b.P = P;
  b.T = T;
  b.plen = plen;
  b.tlen = tlen;
  b.Prev = reversed(P, plen);
  b.Trev = reversed(T, tlen);
  oracle_ws_init(&b.wsf, 1, p->scope);
  oracle_ws_init(&b.wsr, 1, p->scope);
  oracle_ws_init(&b.wsb, 0, p->scope);
  b.score = INT32_MIN; /* cigar_clear() value, kept when nothing sets it */
  int st;
  *ops_len = 0;
  if (p->score_only || ops == NULL) {
    /* wavefront/wavefront_bialign.c:1226-1263 */
    bp_t bp;
    int reached = 0;
    st = find_breakpoint(&b, 0, plen, 0, tlen, C_M, C_M, &bp, &reached);
    if (st == ST_OK || st == ST_END_REACHED) {
      const int s = (st == ST_END_REACHED) ? reached : bp.score;
      *out_score = oracle_classic_score(p, plen, tlen, s);
      st = ST_OK;
    } else {
      *out_score = INT32_MIN;
    }
  } else {
    char* buf = (char*)malloc((size_t)plen + tlen + 8);
    b.ops = buf;
    const int min_length = (plen > tlen ? plen : tlen) <= BI_FALLBACK_MIN_LENGTH;
    st = bi_alignment(&b, 0, plen, 0, tlen, C_M, C_M, min_length ? 0 : INT_MAX, 0);
    if (st == ST_OK) {
      memcpy(ops, buf, (size_t)b.nops);
      *ops_len = b.nops;
    }
    *out_score = b.score;
    free(buf);
  }
  /* cigar->end_v/end_h: the score-only path sets the sequence lengths
   * (wavefront/wavefront_bialign.c:1248-1257), a full alignment only when its
   * top level split at a breakpoint (:1214-1220); a top level that went to the
   * base case appends that CIGAR and keeps the cleared end
   * (:159-194, alignment/cigar.c:79-90) */
  if (end) {
    const int set = (st == ST_OK) && (p->score_only || ops == NULL || b.split0);
    end[0] = set ? plen : -1;
    end[1] = set ? tlen : -1;
  }
  /* wavefront/wavefront_bialign.c:1286-1293 */
  if (st == ST_OK) *out_status = ST_COMPLETED;
  else if (st == ST_MAX_STEPS) *out_status = ST_MAX_STEPS;
  else *out_status = ST_UNATTAINABLE;
  if (cells) *cells = b.cells;
  if (ext) *ext = b.ext;
  oracle_ws_free(&b.wsf);
  oracle_ws_free(&b.wsr);
  oracle_ws_free(&b.wsb);
  free((void*)b.Prev);
  free((void*)b.Trev);
}

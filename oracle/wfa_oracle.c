/*
 * wfa_oracle.c -- CPU restatement of WFA2-lib's exact wavefront alignment
 * (gap-affine and gap-affine-2p, end-to-end, score-only or full CIGAR).
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker the GPU path is compared
 * against.  Nothing in the product library links or calls it.
 *
 * It restates, in plain C and with the reference's own semantics, the
 * unidirectional high-memory algorithm of smarco/WFA2-lib:
 *   - penalty set-up and Eizenga transform  wavefront/wavefront_penalties.c:95-173
 *   - max score scope                        wavefront/wavefront_components.c:81-120
 *   - input fetch (score offsets)            wavefront/wavefront_compute.c:306-352
 *   - output limits                          wavefront/wavefront_compute.c:40-87
 *   - output allocation rule (I/D NULL)      wavefront/wavefront_compute.c:409-494
 *   - compute kernels                        wavefront/wavefront_compute_affine.c:44-86,
 *                                            wavefront/wavefront_compute_affine2p.c:45-106
 *   - end trimming                           wavefront/wavefront_compute.c:579-613
 *   - extend (exact LCP along diagonals)     wavefront/wavefront_extend.c:86-121,
 *                                            wavefront/wavefront_extend_kernels.c:68-123
 *   - end-to-end termination                 wavefront/wavefront_termination.c:37-60
 *   - driver loop, limits, classic score     wavefront/wavefront_unialign.c:98-273,
 *                                            wavefront/wavefront_compute.c:108-120
 *   - backtrace with type priorities        wavefront/wavefront_backtrace.c:36-529
 *
 * The reference pads every input wavefront with NULL offsets beyond its
 * trimmed range [lo,hi] (wavefront/wavefront_compute.c:498-575); here a read
 * outside [lo,hi] simply returns NULL, which is the same value.
 *
 * Memory modes med/low (piggyback back-trace) are reported identical to high
 * on the reference's golden files (tests/wfa.utest.sh:67-78), so they are
 * served by the same high-memory restatement.  Ultralow (BiWFA) is restated
 * in oracle_bialign() below.
 */
#include "wfa_oracle.h"
#include "wfa_oracle_internal.h"

#include <limits.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* wavefront/wavefront_penalties.c:95-173 (Eizenga transform when match<0) */
static int setup_penalties(const int* cfg, pen_t* p) {
  p->metric = cfg[0];
  const int m = cfg[1], x = cfg[2], o1 = cfg[3], e1 = cfg[4], o2 = cfg[5], e2 = cfg[6];
  p->um = m;
  p->ux = x;
  p->uo1 = o1;
  p->ue1 = e1;
  p->uo2 = o2;
  p->ue2 = e2;
  if (p->metric < 0 || p->metric > 4) return -1;
  if (p->metric <= 2) {
    /* wavefront/wavefront_penalties.c:39-94: indel (0), edit (1), gap-linear
     * (2, cfg[3] = the indel penalty; Eizenga transform when match < 0) */
    if (p->metric == 2) {
      if (m > 0 || x <= 0 || o1 <= 0) return -1;
      p->match = m;
      p->x = m < 0 ? 2 * x - 2 * m : x;
      p->o1 = m < 0 ? 2 * o1 - m : o1;
      p->scope = imax(p->x, p->o1) + 1; /* wavefront/wavefront_components.c:63-79 */
    } else {
      p->match = 0;
      p->x = p->metric == 1 ? 1 : -1;
      p->o1 = 1;
      p->scope = 2; /* wavefront/wavefront_components.c:47-61 */
    }
    p->e1 = p->o2 = p->e2 = -1;
  }
  if (p->metric <= 2) goto common;
  if (m > 0 || x <= 0 || o1 < 0 || e1 <= 0) return -1;
  if (p->metric == 4 && (o2 < 0 || e2 <= 0)) return -1;
  if (m < 0) {
    p->match = m;
    p->x = 2 * x - 2 * m;
    p->o1 = 2 * o1;
    p->e1 = 2 * e1 - m;
    p->o2 = 2 * o2;
    p->e2 = 2 * e2 - m;
  } else {
    p->match = 0;
    p->x = x;
    p->o1 = o1;
    p->e1 = e1;
    p->o2 = o2;
    p->e2 = e2;
  }
  if (p->metric == 3) {
    p->o2 = -1;
    p->e2 = -1;
  }
  {
    /* wavefront/wavefront_components.c:81-120 */
    int indel = p->o1 + p->e1;
    if (p->metric == 4) indel = imax(indel, p->o2 + p->e2);
    p->scope = imax(indel, p->x) + 1;
  }
common:
  p->score_only = cfg[8] != 0;
  p->max_steps = cfg[9] > 0 ? cfg[9] : INT_MAX;
  /* wavefront/wavefront_heuristic.c:40-113: cfg[20] is the strategy bit set
   * (cfg[10] == 1 alone is the wf-adaptive shorthand), then its parameters */
  p->heur = cfg[20] != 0 ? cfg[20] : (cfg[10] == 1 ? HS_WFADAPTIVE : 0);
  p->h_min_len = cfg[11];
  p->h_max_dist = cfg[12];
  p->h_steps = cfg[13];
  p->h_xdrop = cfg[21];
  p->h_zdrop = cfg[22];
  p->h_min_k = cfg[23];
  p->h_max_k = cfg[24];
  /* drops with edit/indel: the reference exits (wavefront/wavefront_align.c:83-89) */
  if ((p->heur & (HS_XDROP | HS_ZDROP)) && p->metric <= 1) return -1;
  /* alignment form (wavefront/wavefront_attributes.h:55-69) */
  p->endsfree = cfg[14] == 1;
  p->pbf = cfg[15];
  p->pef = cfg[16];
  p->tbf = cfg[17];
  p->tef = cfg[18];
  p->extension = p->endsfree && cfg[19] != 0;
  if (p->endsfree && (p->pbf < 0 || p->pef < 0 || p->tbf < 0 || p->tef < 0)) return -1;
  /* edit and indel never widen the score-0 wavefront's initialised window
   * [0,0] (wavefront/wavefront_compute_edit.c:321-374), so their back-trace
   * reads begin-free diagonals as sourceless (wavefront/wavefront_backtrace.c:
   * 62-75) and can end in matches over mismatches: a full alignment is not
   * restated.  The score-only search reads the begin-free cells by their
   * limits and is. */
  if (p->endsfree && !p->extension && p->metric <= 1 && (p->pbf > 0 || p->tbf > 0) &&
      !p->score_only)
    return -1;
  return 0;
}

/* Score-only alignments keep only the last max_score_scope scores, as the
 * reference's modular wavefronts do (wavefront/wavefront_compute.c:434-441). */
static orow_t* row_at(oracle_ws_t* ws, int s, int c) {
  if (ws->modular) s %= ws->scope;
  return &ws->rows[(int64_t)s * NCOMP + c];
}

static void ws_ensure_rows(oracle_ws_t* ws, int s) {
  if (ws->modular) s = ws->scope - 1;
  if (s < ws->rows_cap) return;
  int ncap = ws->rows_cap ? ws->rows_cap : 1024;
  while (ncap <= s) ncap *= 2;
  ws->rows = (orow_t*)realloc(ws->rows, (size_t)ncap * NCOMP * sizeof(orow_t));
  memset(ws->rows + (size_t)ws->rows_cap * NCOMP, 0,
         (size_t)(ncap - ws->rows_cap) * NCOMP * sizeof(orow_t));
  ws->rows_cap = ncap;
}

static int32_t* ws_alloc(oracle_ws_t* ws, int64_t n) {
  while (ws->cur < ws->nchunks && ws->chunks[ws->cur].used + n > ws->chunks[ws->cur].cap) ws->cur++;
  if (ws->cur == ws->nchunks) {
    int64_t cap = (int64_t)1 << 20;
    if (ws->nchunks) cap = ws->chunks[ws->nchunks - 1].cap * 2;
    if (cap < n) cap = n;
    ws->chunks = (chunk_t*)realloc(ws->chunks, (size_t)(ws->nchunks + 1) * sizeof(chunk_t));
    ws->chunks[ws->nchunks].mem = (int32_t*)malloc((size_t)cap * sizeof(int32_t));
    ws->chunks[ws->nchunks].cap = cap;
    ws->chunks[ws->nchunks].used = 0;
    ws->nchunks++;
  }
  chunk_t* c = &ws->chunks[ws->cur];
  int32_t* p = c->mem + c->used;
  c->used += n;
  return p;
}

static void ws_reset(oracle_ws_t* ws) {
  for (int i = 0; i < ws->nchunks; ++i) ws->chunks[i].used = 0;
  ws->cur = 0;
}

/* Grows a k-indexed buffer to cover [lo,hi]; NULL-fills it when fill is set. */
static void kbuf_cover(kbuf_t* b, int lo, int hi, int fill) {
  if (b->mem && b->lo <= lo && hi <= b->hi) return;
  const int nlo = b->mem ? imin(lo, b->lo) - 256 : lo - 256;
  const int nhi = b->mem ? imax(hi, b->hi) + 256 : hi + 256;
  free(b->mem);
  b->mem = (int32_t*)malloc((size_t)(nhi - nlo + 1) * sizeof(int32_t));
  if (fill)
    for (int i = 0; i <= nhi - nlo; ++i) b->mem[i] = WF_NULL;
  b->lo = nlo;
  b->hi = nhi;
}
static int32_t* kbuf_at0(kbuf_t* b) { return b->mem - b->lo; }

/* Storage for row (s,c) over diagonals [lo,hi] (k-indexed pointer). */
static int32_t* row_storage(oracle_ws_t* ws, int s, int c, int lo, int hi) {
  if (!ws->modular) return ws_alloc(ws, hi - lo + 1) - lo;
  kbuf_t* b = &ws->slotbuf[(s % ws->scope) * NCOMP + c];
  kbuf_cover(b, lo, hi, 0);
  return kbuf_at0(b);
}

static void ws_free(oracle_ws_t* ws) {
  for (int i = 0; i < ws->nchunks; ++i) free(ws->chunks[i].mem);
  free(ws->chunks);
  free(ws->rows);
  free(ws->nullbuf.mem);
  free(ws->victim.mem);
  if (ws->slotbuf) {
    for (int i = 0; i < ws->scope * NCOMP; ++i) free(ws->slotbuf[i].mem);
    free(ws->slotbuf);
  }
}

/* wavefront/wavefront_compute.c:354-368: NULL or null wavefronts read as the
 * shared all-NULL wavefront (lo=1, hi=-1; wavefront/wavefront.c:118-145). */
static orow_t* fetch(oracle_ws_t* ws, orow_t* nullrow, int s, int c) {
  if (s < 0) return nullrow;
  orow_t* r = row_at(ws, s, c);
  if (!r->exists || r->null) return nullrow;
  return r;
}

/* wavefront/wavefront_compute.c:498-527: NULL-pad an input beyond its
 * initialised window so the compute loop reads [lo,hi] without peeling. */
static void init_ends(orow_t* r, int lo, int hi) {
  if (r->null) return;
  /* the pad starts beyond both the window and the limits: an ends-free
   * start keeps the window [0,0] inside wider limits */
  if (r->ilo > lo) {
    const int end = imin(r->ilo, r->lo);
    for (int k = lo; k < end; ++k) r->off[k] = WF_NULL;
    r->ilo = lo;
  }
  if (r->ihi < hi) {
    const int start = imax(r->ihi, r->hi) + 1;
    for (int k = start; k <= hi; ++k) r->off[k] = WF_NULL;
    r->ihi = hi;
  }
}

/* Ends-free with match < 0: the begin-free diagonals enter one at a time, at
 * the scores that are multiples of -match (wavefront/wavefront_compute.c:
 * 124-145).  Returns that diagonal (and which sides are free), or -1. */
static int endsfree_k_of(const pen_t* p, int endsfree, int s, int* text_free,
                         int* pattern_free) {
  if (!endsfree || p->match == 0 || p->extension) return -1;
  if (p->pbf == 0 && p->tbf == 0) return -1;
  if (s % (-p->match) != 0) return -1;
  const int ek = s / (-p->match);
  *text_free = p->tbf >= ek;
  *pattern_free = p->pbf >= ek;
  return (*text_free || *pattern_free) ? ek : -1;
}

/* The begin cells (0,ek) and (ek,0) enter the computed M wavefront when they
 * lie ahead of it (wavefront/wavefront_compute.c:173-215), before trimming. */
static void endsfree_init(orow_t* r, int ek, int text_free, int pattern_free) {
  const int lo = r->lo, hi = r->hi;
  if (text_free) {
    if (hi >= ek) {
      if (r->off[ek] <= ek) r->off[ek] = ek;
    } else {
      for (int k = hi + 1; k < ek; ++k) r->off[k] = WF_NULL;
      r->off[ek] = ek;
      r->hi = ek;
    }
  }
  if (pattern_free) {
    const int k0 = -ek;
    if (lo <= k0) {
      if (r->off[k0] <= 0) r->off[k0] = 0;
    } else {
      r->off[k0] = 0;
      for (int k = k0 + 1; k < lo; ++k) r->off[k] = WF_NULL;
      r->lo = k0;
    }
  }
}

/* A null step that still holds begin cells: an M wavefront of only those
 * (wavefront/wavefront_compute.c:217-262), untrimmed. */
static void endsfree_null_row(oracle_ws_t* ws, const pen_t* p, int s, int ek, int text_free,
                              int pattern_free) {
  const int lo = pattern_free ? -ek : ek, hi = text_free ? ek : -ek;
  ws->hlo = imin(ws->hlo, lo - (p->scope + 1));
  ws->hhi = imax(ws->hhi, hi + (p->scope + 1));
  kbuf_cover(&ws->nullbuf, ws->hlo, ws->hhi, 1);
  kbuf_cover(&ws->victim, ws->hlo, ws->hhi, 0);
  orow_t* r = row_at(ws, s, C_M);
  r->off = row_storage(ws, s, C_M, ws->hlo, ws->hhi);
  r->exists = 1;
  r->null = 0;
  r->lo = r->ilo = lo;
  r->hi = r->ihi = hi;
  for (int k = lo; k <= hi; ++k) r->off[k] = WF_NULL;
  if (text_free) r->off[ek] = ek;
  if (pattern_free) r->off[-ek] = 0;
}

/* wavefront/wavefront_compute.c:579-613 */
static void trim_row(orow_t* r, int plen, int tlen) {
  int k;
  for (k = r->hi; k >= r->lo; --k) {
    const int32_t off = r->off[k];
    if ((uint32_t)off <= (uint32_t)tlen && (uint32_t)(off - k) <= (uint32_t)plen) break;
  }
  r->hi = k;
  r->ihi = k;
  const int hi = r->hi;
  for (k = r->lo; k <= hi; ++k) {
    const int32_t off = r->off[k];
    if ((uint32_t)off <= (uint32_t)tlen && (uint32_t)(off - k) <= (uint32_t)plen) break;
  }
  r->lo = k;
  r->ilo = k;
  r->null = (r->lo > r->hi);
}

/* Edit-distance exact pruning of an end-to-end wavefront of at least 1000
 * diagonals (wavefront/wavefront_compute_edit.c:199-279): diagonals whose
 * best case (|k - k_end| edits left) exceeds the best worst case (the larger
 * remainder) of any diagonal are dropped from the limits. */
static void edit_exact_prune(orow_t* r, int plen, int tlen) {
  const int lo = r->lo, hi = r->hi;
  if (hi - lo + 1 < 1000) return;
  const int k_end = tlen - plen;
  const int sample_k = lo + (hi - lo) / 2;
  const int32_t so = r->off[sample_k];
  if (so < 0) return;
  const int smax_sample = imax(plen - (so - sample_k), tlen - so);
  const int smin_lo = lo - k_end >= 0 ? lo - k_end : k_end - lo;
  const int smin_hi = hi - k_end >= 0 ? hi - k_end : k_end - hi;
  if (smin_lo <= smax_sample && smin_hi <= smax_sample) return;
  int wmin = INT_MAX;
  for (int k = lo; k <= hi; ++k) {
    const int32_t off = r->off[k];
    if (off < 0) continue;
    const int w = imax(plen - (off - k), tlen - off);
    if (w < wmin) wmin = w;
  }
  /* the best case |(plen - v) - (tlen - h)| = |k - k_end| for any offset */
  int nlo = lo;
  for (int k = lo; k <= hi; ++k) {
    const int b = k - k_end >= 0 ? k - k_end : k_end - k;
    if (b <= wmin) break;
    ++nlo;
  }
  int nhi = hi;
  for (int k = hi; k > nlo; --k) {
    const int b = k - k_end >= 0 ? k - k_end : k_end - k;
    if (b <= wmin) break;
    --nhi;
  }
  r->lo = nlo;
  r->hi = nhi;
}

/* One compute step of the single-component metrics (indel, edit, gap-linear):
 * wavefront/wavefront_compute_edit.c:321-374 (indel/edit: M[s-1] only, limits
 * one wider, the two elements beyond each end of M[s-1] NULLed, a null result
 * ends the alignment, end-to-end edit pruned) and
 * wavefront/wavefront_compute_linear.c:168-197 (gap-linear: M[s-x], M[s-o]).
 * Returns cells computed. */
static int64_t compute_step_linear(oracle_ws_t* ws, const pen_t* p, int s, int plen, int tlen,
                                   int* null_steps, int endsfree) {
  ws_ensure_rows(ws, s);
  orow_t nullrow = {.exists = 1, .null = 1, .lo = 1, .hi = -1, .ilo = 1, .ihi = -1, .off = kbuf_at0(&ws->nullbuf)};
  const int editlike = p->metric <= 1;
  orow_t* mx = editlike ? (p->metric == 1 ? fetch(ws, &nullrow, s - 1, C_M) : &nullrow)
                        : fetch(ws, &nullrow, s - p->x, C_M);
  orow_t* mo = fetch(ws, &nullrow, s - p->o1, C_M);
  for (int c = 0; c < NCOMP; ++c) memset(row_at(ws, s, c), 0, sizeof(orow_t));
  int lo, hi;
  if (editlike) {
    if (mo->null) {  /* wavefront/wavefront_compute_edit.c:372 */
      *null_steps = INT_MAX / 2;
      return 0;
    }
    lo = mo->lo - 1;
    hi = mo->hi + 1;
  } else {
    if (mx->null && mo->null) {
      (*null_steps)++;
      int tf, pf;
      const int ek = endsfree_k_of(p, endsfree, s, &tf, &pf);
      if (ek >= 0) endsfree_null_row(ws, p, s, ek, tf, pf);
      return 0;
    }
    *null_steps = 0;
    lo = imin(mx->lo, mo->lo - 1);
    hi = imax(mx->hi, mo->hi + 1);
  }
  int tf = 0, pf = 0;
  const int ek = editlike ? -1 : endsfree_k_of(p, endsfree, s, &tf, &pf);
  /* the allocation also covers the begin cells (wavefront/wavefront_compute.c:419-428) */
  const int alo = (ek >= 0 && pf) ? imin(lo, -ek) : lo, ahi = (ek >= 0 && tf) ? imax(hi, ek) : hi;
  ws->hlo = imin(ws->hlo, alo - (p->scope + 1));
  ws->hhi = imax(ws->hhi, ahi + (p->scope + 1));
  kbuf_cover(&ws->nullbuf, ws->hlo, ws->hhi, 1);
  kbuf_cover(&ws->victim, ws->hlo, ws->hhi, 0);
  nullrow.off = kbuf_at0(&ws->nullbuf);
  if (editlike) {
    mo->off[lo - 1] = WF_NULL;
    mo->off[lo] = WF_NULL;
    mo->off[hi] = WF_NULL;
    mo->off[hi + 1] = WF_NULL;
  } else {
    init_ends(mx, lo, hi);
    init_ends(mo, lo - 1, hi + 1);
  }
  orow_t* r = row_at(ws, s, C_M);
  r->off = row_storage(ws, s, C_M, ws->hlo, ws->hhi);
  r->exists = 1;
  r->lo = r->ilo = lo;
  r->hi = r->ihi = hi;
  const int32_t* const m_x = (editlike && p->metric == 1) ? mo->off : mx->off;
  const int32_t* const m_o = mo->off;
  int32_t* const o_m = r->off;
  for (int k = lo; k <= hi; ++k) {
    /* wavefront/wavefront_compute_edit.c:44-93, wavefront/wavefront_compute_linear.c:45-66 */
    int32_t mmax;
    if (p->metric == 0) {
      const int32_t ins = m_o[k - 1] + 1, del = m_o[k + 1];
      mmax = del > ins ? del : ins;
    } else {
      const int32_t ins = m_o[k - 1], misms = m_x[k], del = m_o[k + 1];
      const int32_t im = (misms > ins ? misms : ins) + 1;
      mmax = del > im ? del : im;
    }
    if ((uint32_t)mmax > (uint32_t)tlen) mmax = WF_NULL;
    if ((uint32_t)(mmax - k) > (uint32_t)plen) mmax = WF_NULL;
    o_m[k] = mmax;
  }
  if (ek >= 0) endsfree_init(r, ek, tf, pf);
  trim_row(r, plen, tlen);
  if (editlike) {
    if (r->null) *null_steps = INT_MAX / 2;
    if (p->metric == 1 && !endsfree && !r->null) edit_exact_prune(r, plen, tlen);
  }
  return hi - lo + 1;
}

/* One compute step at score s (wavefront/wavefront_compute_affine.c:229-260 and
 * wavefront/wavefront_compute_affine2p.c:322-360).  Returns cells computed. */
static int64_t compute_step(oracle_ws_t* ws, const pen_t* p, int s, int plen, int tlen,
                            int* null_steps, int endsfree) {
  if (p->metric <= 2) return compute_step_linear(ws, p, s, plen, tlen, null_steps, endsfree);
  const int a2p = (p->metric == 4);
  ws_ensure_rows(ws, s);
  orow_t nullrow = {.exists = 1, .null = 1, .lo = 1, .hi = -1, .ilo = 1, .ihi = -1, .off = kbuf_at0(&ws->nullbuf)};
  orow_t* mx = fetch(ws, &nullrow, s - p->x, C_M);
  orow_t* mo1 = fetch(ws, &nullrow, s - p->o1 - p->e1, C_M);
  orow_t* i1e = fetch(ws, &nullrow, s - p->e1, C_I1);
  orow_t* d1e = fetch(ws, &nullrow, s - p->e1, C_D1);
  orow_t* mo2 = &nullrow;
  orow_t* i2e = &nullrow;
  orow_t* d2e = &nullrow;
  if (a2p) {
    mo2 = fetch(ws, &nullrow, s - p->o2 - p->e2, C_M);
    i2e = fetch(ws, &nullrow, s - p->e2, C_I2);
    d2e = fetch(ws, &nullrow, s - p->e2, C_D2);
  }
  for (int c = 0; c < NCOMP; ++c) memset(row_at(ws, s, c), 0, sizeof(orow_t));
  if (mx->null && mo1->null && i1e->null && d1e->null && mo2->null && i2e->null && d2e->null) {
    (*null_steps)++;
    int tf, pf;
    const int ek = endsfree_k_of(p, endsfree, s, &tf, &pf);
    if (ek >= 0) endsfree_null_row(ws, p, s, ek, tf, pf);
    return 0;
  }
  *null_steps = 0;
  /* wavefront/wavefront_compute.c:40-87 (null rows carry lo=1,hi=-1) */
  int lo = mx->lo, hi = mx->hi;
  lo = imin(lo, mo1->lo - 1);
  hi = imax(hi, mo1->hi + 1);
  lo = imin(lo, i1e->lo + 1);
  hi = imax(hi, i1e->hi + 1);
  lo = imin(lo, d1e->lo - 1);
  hi = imax(hi, d1e->hi - 1);
  if (a2p) {
    lo = imin(lo, mo2->lo - 1);
    hi = imax(hi, mo2->hi + 1);
    lo = imin(lo, i2e->lo + 1);
    hi = imax(hi, i2e->hi + 1);
    lo = imin(lo, d2e->lo - 1);
    hi = imax(hi, d2e->hi - 1);
  }
  /* wavefront/wavefront_compute.c:88-104: allocation padded by scope+1 and
   * never narrower than any earlier allocation of the alignment; it also
   * covers ends-free begin cells (:419-428) */
  int tf = 0, pf = 0;
  const int ek = endsfree_k_of(p, endsfree, s, &tf, &pf);
  const int elo = (ek >= 0 && pf) ? imin(lo, -ek) : lo, ehi = (ek >= 0 && tf) ? imax(hi, ek) : hi;
  ws->hlo = imin(ws->hlo, elo - (p->scope + 1));
  ws->hhi = imax(ws->hhi, ehi + (p->scope + 1));
  kbuf_cover(&ws->nullbuf, ws->hlo, ws->hhi, 1);
  kbuf_cover(&ws->victim, ws->hlo, ws->hhi, 0);
  nullrow.off = kbuf_at0(&ws->nullbuf);
  const int alo = ws->hlo, awidth = ws->hhi - ws->hlo + 1;
  /* wavefront/wavefront_compute.c:447-492: I/D outputs exist only if an input does */
  const int has[NCOMP] = {1, (!mo1->null || !i1e->null), (!mo1->null || !d1e->null),
                          a2p && (!mo2->null || !i2e->null), a2p && (!mo2->null || !d2e->null)};
  int32_t* out[NCOMP];
  int32_t* const victim = kbuf_at0(&ws->victim);
  for (int c = 0; c < NCOMP; ++c) {
    orow_t* r = row_at(ws, s, c);
    out[c] = victim;
    if (has[c]) {
      r->off = row_storage(ws, s, c, alo, alo + awidth - 1);
      r->exists = 1;
      r->lo = lo;
      r->hi = hi;
      r->ilo = lo;
      r->ihi = hi;
      out[c] = r->off;
    }
  }
  /* wavefront/wavefront_compute.c:528-575 */
  init_ends(mx, lo, hi);
  init_ends(mo1, lo - 1, hi + 1);
  init_ends(i1e, lo - 1, hi);
  init_ends(d1e, lo, hi + 1);
  if (a2p) {
    init_ends(mo2, lo - 1, hi + 1);
    init_ends(i2e, lo - 1, hi);
    init_ends(d2e, lo, hi + 1);
  }
  const int32_t* __restrict__ const m_x = mx->off;
  const int32_t* __restrict__ const m_o1 = mo1->off;
  const int32_t* __restrict__ const i_e1 = i1e->off;
  const int32_t* __restrict__ const d_e1 = d1e->off;
  int32_t* __restrict__ const o_m = out[C_M];
  int32_t* __restrict__ const o_i1 = out[C_I1];
  int32_t* __restrict__ const o_d1 = out[C_D1];
  if (!a2p) {
    /* wavefront/wavefront_compute_affine.c:65-85 (the reference vectorises
     * this loop with PRAGMA_LOOP_VECTORIZE, utils/commons.h:252-256) */
#pragma GCC ivdep
    for (int k = lo; k <= hi; ++k) {
      const int32_t ins1 = (m_o1[k - 1] > i_e1[k - 1] ? m_o1[k - 1] : i_e1[k - 1]) + 1;
      const int32_t del1 = m_o1[k + 1] > d_e1[k + 1] ? m_o1[k + 1] : d_e1[k + 1];
      o_i1[k] = ins1;
      o_d1[k] = del1;
      const int32_t misms = m_x[k] + 1;
      int32_t mmax = misms > ins1 ? misms : ins1;
      mmax = del1 > mmax ? del1 : mmax;
      if ((uint32_t)mmax > (uint32_t)tlen) mmax = WF_NULL;
      if ((uint32_t)(mmax - k) > (uint32_t)plen) mmax = WF_NULL;
      o_m[k] = mmax;
    }
  } else {
    /* wavefront/wavefront_compute_affine2p.c:71-105 */
    const int32_t* __restrict__ const m_o2 = mo2->off;
    const int32_t* __restrict__ const i_e2 = i2e->off;
    const int32_t* __restrict__ const d_e2 = d2e->off;
    int32_t* __restrict__ const o_i2 = out[C_I2];
    int32_t* __restrict__ const o_d2 = out[C_D2];
#pragma GCC ivdep
    for (int k = lo; k <= hi; ++k) {
      const int32_t ins1 = (m_o1[k - 1] > i_e1[k - 1] ? m_o1[k - 1] : i_e1[k - 1]) + 1;
      const int32_t ins2 = (m_o2[k - 1] > i_e2[k - 1] ? m_o2[k - 1] : i_e2[k - 1]) + 1;
      const int32_t del1 = m_o1[k + 1] > d_e1[k + 1] ? m_o1[k + 1] : d_e1[k + 1];
      const int32_t del2 = m_o2[k + 1] > d_e2[k + 1] ? m_o2[k + 1] : d_e2[k + 1];
      o_i1[k] = ins1;
      o_i2[k] = ins2;
      o_d1[k] = del1;
      o_d2[k] = del2;
      const int32_t ins = ins1 > ins2 ? ins1 : ins2;
      const int32_t del = del1 > del2 ? del1 : del2;
      const int32_t misms = m_x[k] + 1;
      int32_t mmax = misms > ins ? misms : ins;
      mmax = del > mmax ? del : mmax;
      if ((uint32_t)mmax > (uint32_t)tlen) mmax = WF_NULL;
      if ((uint32_t)(mmax - k) > (uint32_t)plen) mmax = WF_NULL;
      o_m[k] = mmax;
    }
  }
  /* wavefront/wavefront_compute.c:614-633: begin cells, then trimming */
  if (ek >= 0) endsfree_init(row_at(ws, s, C_M), ek, tf, pf);
  for (int c = 0; c < NCOMP; ++c) {
    orow_t* r = row_at(ws, s, c);
    if (r->exists) trim_row(r, plen, tlen);
  }
  return hi - lo + 1;
}

/* Exact LCP along a diagonal, stopping at the sequence ends
 * (wavefront/wavefront_extend_kernels.c:68-92; the reference stops on the EOS
 * sentinels of wavefront/wavefront_sequences.c:37-39). */
static inline int lcp(const char* P, int plen, const char* T, int tlen, int v, int h) {
  int n = 0;
  const int lim = imin(plen - v, tlen - h);
  while (n + 8 <= lim) {
    uint64_t a, b;
    memcpy(&a, P + v + n, 8);
    memcpy(&b, T + h + n, 8);
    const uint64_t d = a ^ b;
    if (d) {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
      return n + (__builtin_ctzll(d) >> 3);
#else
      break;
#endif
    }
    n += 8;
  }
  while (n < lim && P[v + n] == T[h + n]) ++n;
  return n;
}

/* wavefront/wavefront_backtrace.c:36-59: (offset<<4)|type, larger wins */
enum { BT_M = 9, BT_D2E = 8, BT_D2O = 7, BT_D1E = 6, BT_D1O = 5, BT_I2E = 4, BT_I2O = 3, BT_I1E = 2, BT_I1O = 1 };

static inline int64_t cand(oracle_ws_t* ws, int s, int c, int k, int add, int type) {
  if (s < 0) return WF_NULL;
  const orow_t* r = row_at(ws, s, c);
  if (!r->exists || k < r->ilo || k > r->ihi) return WF_NULL;
  return ((int64_t)(r->off[k] + add) << 4) | type;
}
static inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }

/* wavefront/wavefront_backtrace.c:320-529, writing into a reversed buffer.
 * Returns the number of operations, or -1 on an inconsistent trace. */
#define PUT(c)            \
  do {                    \
    if (n >= cap) return -1; \
    rev[n++] = (c);       \
  } while (0)
/* wavefront/wavefront_backtrace.c:76-100 moves the CIGAR's begin by the
 * count first: a negative count (a source ahead of the cell, read from a
 * wavefront a cut emptied) takes back that many operations */
#define MATCHES(cnt)                               \
  do {                                             \
    const int nm_ = (cnt);                         \
    if (nm_ < 0) {                                 \
      n += nm_;                                    \
      if (n < 0) return -1;                        \
    } else {                                       \
      for (int i_ = 0; i_ < nm_; ++i_) PUT('M');   \
    }                                              \
  } while (0)
static int backtrace(oracle_ws_t* ws, const pen_t* p, int plen, int tlen, int score, int k_end,
                     int32_t off_end, int comp_end, char* rev, int cap, int* stale) {
  int n = 0;
  int mat = comp_end;
  int s = score, k = k_end;
  int32_t offset = off_end;
  int h = offset, v = offset - k;
  const int a2p = (p->metric == 4);
  /* ending deletions, then insertions: the free end of an ends-free alignment
   * (wavefront/wavefront_backtrace.c:346-356); none end-to-end (v==plen, h==tlen) */
  if (comp_end == C_M) {
    for (int i = plen - v; i > 0; --i) PUT('D');
    for (int i = tlen - h; i > 0; --i) PUT('I');
  }
  while (v > 0 && h > 0 && s > 0) {
    const int sx = s - p->x, so1 = s - p->o1 - p->e1, so2 = s - p->o2 - p->e2;
    const int se1 = s - p->e1, se2 = s - p->e2;
    int64_t mall;
    if (p->metric <= 2) {
      /* wavefront/wavefront_backtrace.c:223-319: one component; the gap
       * candidates read M[s - gap_opening1] */
      const int sg = s - p->o1;
      const int64_t misms = p->metric != 0 ? cand(ws, sx, C_M, k, 1, BT_M) : WF_NULL;
      mall = max64(misms, max64(cand(ws, sg, C_M, k - 1, 1, BT_I1O), cand(ws, sg, C_M, k + 1, 0, BT_D1O)));
      if (mall < 0) break;
      const int moff = (int)(mall >> 4);
      MATCHES(offset - moff);
      offset = moff;
      v = offset - k;
      h = offset;
      if (v <= 0 || h <= 0) break;
      const int type = (int)(mall & 0xF);
      if (type == BT_M) { s = sx; PUT('X'); --offset; }
      else if (type == BT_I1O) { s = sg; PUT('I'); --k; --offset; }
      else { s = sg; PUT('D'); ++k; }
      if (row_at(ws, s, C_M)->cut_null) *stale = 1;
      v = offset - k;
      h = offset;
      continue;
    }
    switch (mat) {
      case C_M: {
        const int64_t misms = cand(ws, sx, C_M, k, 1, BT_M);
        const int64_t i1 = max64(cand(ws, so1, C_M, k - 1, 1, BT_I1O), cand(ws, se1, C_I1, k - 1, 1, BT_I1E));
        const int64_t d1 = max64(cand(ws, so1, C_M, k + 1, 0, BT_D1O), cand(ws, se1, C_D1, k + 1, 0, BT_D1E));
        if (!a2p) {
          mall = max64(misms, max64(i1, d1));
        } else {
          const int64_t i2 = max64(cand(ws, so2, C_M, k - 1, 1, BT_I2O), cand(ws, se2, C_I2, k - 1, 1, BT_I2E));
          const int64_t d2 = max64(cand(ws, so2, C_M, k + 1, 0, BT_D2O), cand(ws, se2, C_D2, k + 1, 0, BT_D2E));
          mall = max64(misms, max64(max64(i1, i2), max64(d1, d2)));
        }
        break;
      }
      case C_I1:
        mall = max64(cand(ws, so1, C_M, k - 1, 1, BT_I1O), cand(ws, se1, C_I1, k - 1, 1, BT_I1E));
        break;
      case C_I2:
        mall = max64(cand(ws, so2, C_M, k - 1, 1, BT_I2O), cand(ws, se2, C_I2, k - 1, 1, BT_I2E));
        break;
      case C_D1:
        mall = max64(cand(ws, so1, C_M, k + 1, 0, BT_D1O), cand(ws, se1, C_D1, k + 1, 0, BT_D1E));
        break;
      default: /* C_D2 */
        mall = max64(cand(ws, so2, C_M, k + 1, 0, BT_D2O), cand(ws, se2, C_D2, k + 1, 0, BT_D2E));
        break;
    }
    if (mall < 0) break;
    if (mat == C_M) {
      const int moff = (int)(mall >> 4);
      MATCHES(offset - moff);
      offset = moff;
      v = offset - k;
      h = offset;
      if (v <= 0 || h <= 0) break;
    }
    const int type = (int)(mall & 0xF);
    switch (type) {
      case BT_M: s = sx; mat = C_M; break;
      case BT_I1O: s = so1; mat = C_M; break;
      case BT_I1E: s = se1; mat = C_I1; break;
      case BT_I2O: s = so2; mat = C_M; break;
      case BT_I2E: s = se2; mat = C_I2; break;
      case BT_D1O: s = so1; mat = C_M; break;
      case BT_D1E: s = se1; mat = C_D1; break;
      case BT_D2O: s = so2; mat = C_M; break;
      case BT_D2E: s = se2; mat = C_D2; break;
      default: return -1;
    }
    if (row_at(ws, s, mat)->cut_null) *stale = 1;
    switch (type) {
      case BT_M: PUT('X'); --offset; break;
      case BT_I1O: case BT_I1E: case BT_I2O: case BT_I2E: PUT('I'); --k; --offset; break;
      default: PUT('D'); ++k; break;
    }
    v = offset - k;
    h = offset;
  }
  if (mat == C_M) {
    if (v > 0 && h > 0) {
      const int nm = imin(v, h);
      for (int i = 0; i < nm; ++i) PUT('M');
      v -= nm;
      h -= nm;
    }
    while (v > 0) { PUT('D'); --v; }
    while (h > 0) { PUT('I'); --h; }
  } else if (v != 0 || h != 0 || (s != 0 && p->match == 0)) {
    return -1;
  }
  return n;
}
#undef PUT
#undef MATCHES

/* wavefront/wavefront_compute.c:108-120 (edit and indel: the distance) */
static int classic_score(const pen_t* p, int plen, int tlen, int s) {
  if (p->metric <= 1) return s;
  if (p->match == 0) return -s;
  const int swg_match = -p->match;
  return (swg_match * (plen + tlen) - s) / 2;
}

/* classic_score in the reference's int arithmetic, which wraps for the NULL
 * end position of an alignment that ran out of wavefronts */
static int classic_score_wrapped(const pen_t* p, int v, int h, int s) {
  if (p->metric <= 1) return s;
  if (p->match == 0) return -s;
  const uint32_t sum = (uint32_t)v + (uint32_t)h;
  return (int)((uint32_t)(-p->match) * sum - (uint32_t)s) / 2;
}

/* One unidirectional alignment (wavefront/wavefront_unialign.c:242-273). */
const orow_t* oracle_row(oracle_ws_t* ws, int s, int c) { return row_at(ws, s, c); }

void oracle_ws_init(oracle_ws_t* ws, int modular, int scope) {
  memset(ws, 0, sizeof(*ws));
  ws->modular = modular;
  ws->scope = scope;
  if (modular) ws->slotbuf = (kbuf_t*)calloc((size_t)scope * NCOMP, sizeof(kbuf_t));
}

void oracle_ws_free(oracle_ws_t* ws) { ws_free(ws); }

/* ------------------------------------------------------------- stepper */
/* Score-0 wavefront for an alignment that begins in component cb
 * (wavefront/wavefront_aligner.c:236-382): M[0][0]=0, or the gap component's
 * offset 0 on diagonal 0 with no M wavefront. */
void oracle_ua_start(oracle_ua_t* ua, oracle_ws_t* ws, const pen_t* p, const char* P, int plen,
                     const char* T, int tlen, int cb, int ce) {
  ua->ws = ws;
  ua->p = p;
  ua->P = P;
  ua->plen = plen;
  ua->T = T;
  ua->tlen = tlen;
  ua->cb = cb;
  ua->ce = ce;
  ua->s = 0;
  ua->null_steps = 0;
  ua->k_end = tlen - plen;
  ua->cells = 0;
  ua->ext = 0;
  ua->heur = p->heur;
  ua->steps_wait = p->h_steps;
  ua->max_sw = 0;
  ua->max_sw_k = INT32_MAX; /* DPMATRIX_DIAGONAL_NULL */
  ua->max_sw_off = WF_NULL;
  ua->max_wf_score = -1;
  ua->zdropped = 0;
  ua->stale_source = 0;
  ua->endsfree = 0;
  ua->pbf = ua->pef = ua->tbf = ua->tef = 0;
  ua->end_k = tlen - plen;
  ua->end_off = tlen;
  ws_reset(ws);
  ws_ensure_rows(ws, 0);
  if (ws->modular) memset(ws->rows, 0, (size_t)ws->scope * NCOMP * sizeof(orow_t));
  for (int c = 0; c < NCOMP; ++c) memset(row_at(ws, 0, c), 0, sizeof(orow_t));
  /* allocation padded as wavefront_compute_limits_output does
   * (wavefront/wavefront_compute.c:88-104) */
  ws->hlo = -(p->scope + 1);
  ws->hhi = p->scope + 1;
  kbuf_cover(&ws->nullbuf, ws->hlo, ws->hhi, 1);
  kbuf_cover(&ws->victim, ws->hlo, ws->hhi, 0);
  orow_t* r0 = row_at(ws, 0, cb);
  r0->off = row_storage(ws, 0, cb, ws->hlo, ws->hhi);
  r0->exists = 1;
  r0->lo = r0->hi = r0->ilo = r0->ihi = 0;
  r0->off[0] = 0;
}

/* Ends-free start (wavefront/wavefront_aligner.c:250-305): with match 0 the
 * score-0 M wavefront spans [-pattern_begin_free, text_begin_free], diagonal
 * k > 0 starting at (v,h) = (0,k) and k < 0 at (-k,0).  Its initialised window
 * stays [0,0]: compute steps NULL-pad only beyond min/max(window, limits)
 * (wavefront/wavefront_compute.c:498-527), so cells a heuristic cut from the
 * limits before the first such pad are NULLed by it. */
void oracle_ua_start_endsfree(oracle_ua_t* ua, oracle_ws_t* ws, const pen_t* p, const char* P,
                              int plen, const char* T, int tlen, int pbf, int pef, int tbf,
                              int tef) {
  oracle_ua_start(ua, ws, p, P, plen, T, tlen, C_M, C_M);
  ua->endsfree = 1;
  ua->pbf = pbf;
  ua->pef = pef;
  ua->tbf = tbf;
  ua->tef = tef;
  const int lo = p->match == 0 ? -pbf : 0;
  const int hi = p->match == 0 ? tbf : 0;
  if (lo == 0 && hi == 0) return;
  ws_reset(ws);
  ws->hlo = lo - (p->scope + 1);
  ws->hhi = hi + p->scope + 1;
  kbuf_cover(&ws->nullbuf, ws->hlo, ws->hhi, 1);
  kbuf_cover(&ws->victim, ws->hlo, ws->hhi, 0);
  orow_t* r0 = row_at(ws, 0, C_M);
  r0->off = row_storage(ws, 0, C_M, ws->hlo, ws->hhi);
  r0->exists = 1;
  r0->null = 0;
  r0->lo = lo;
  r0->hi = hi;
  r0->ilo = r0->ihi = 0;
  for (int k = lo; k <= hi; ++k) r0->off[k] = k > 0 ? k : 0;
}

/* Wrapping int32 arithmetic: the reference computes these differences in
 * int, where the NULL offsets and an INT_MIN maximum can overflow. */
static int wsub(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }

/* Distance of a cell to the end (wavefront/wavefront_heuristic.c:125-145);
 * wfmash weighs each side by its length. */
static int hs_distance(const oracle_ua_t* ua, int k, int32_t off, int wfmash) {
  if (off < 0) return -WF_NULL;
  const int plen = ua->plen, tlen = ua->tlen;
  const int v = off - k, h = off;
  if (!wfmash) return imax(plen - v, tlen - h);
  const int mfactor = (int)((float)(plen + tlen) / 2);
  const int left_v = (int)((float)(plen - v) / plen * mfactor);
  const int left_h = (int)((float)(tlen - h) / tlen * mfactor);
  return imax(left_v, left_h);
}

/* wf-adaptive and wfmash (wavefront/wavefront_heuristic.c:229-289): cells
 * further than max_distance_threshold beyond the closest are cut from both
 * ends, keeping the end diagonal's side. */
static void hs_wfadaptive(oracle_ua_t* ua, orow_t* m, int wfmash) {
  const pen_t* p = ua->p;
  if (ua->steps_wait > 0) return;
  const int lo = m->lo, hi = m->hi;
  if (hi - lo + 1 < p->h_min_len) return;
  int* dist = (int*)malloc((size_t)(hi - lo + 1) * sizeof(int));
  int min_d = imax(ua->plen, ua->tlen);
  for (int k = lo; k <= hi; ++k) {
    dist[k - lo] = hs_distance(ua, k, m->off[k], wfmash);
    min_d = imin(min_d, dist[k - lo]);
  }
  const int k_a = ua->tlen - ua->plen;
  const int top = imin(k_a, hi);
  int nlo = lo;
  for (int k = lo; k < top; ++k) {
    if (dist[k - lo] - min_d <= p->h_max_dist) break;
    ++nlo;
  }
  const int bot = imax(k_a, nlo);
  int nhi = hi;
  for (int k = hi; k > bot; --k) {
    if (dist[k - lo] - min_d <= p->h_max_dist) break;
    --nhi;
  }
  free(dist);
  m->lo = nlo;
  m->hi = nhi;
  ua->steps_wait = p->h_steps;
}

/* SW-style score of every cell (wavefront/wavefront_heuristic.c:294-325,
 * wavefront/wavefront_penalties.h:73) and the first maximum. */
static int* hs_sw_scores(const oracle_ua_t* ua, const orow_t* m, int* cmax, int* cmax_k,
                         int32_t* cmax_off) {
  const int swg = ua->p->match != 0 ? -ua->p->match : -1;
  int* sw = (int*)malloc((size_t)(m->hi - m->lo + 1) * sizeof(int));
  *cmax = INT_MIN;
  *cmax_k = 0;
  *cmax_off = 0;
  for (int k = m->lo; k <= m->hi; ++k) {
    const int32_t off = m->off[k];
    if (off < 0) continue;
    const int v = off - k, h = off;
    const int sc = (swg * (v + h) - ua->s) / 2;
    sw[k - m->lo] = sc;
    if (*cmax < sc) {
      *cmax = sc;
      *cmax_k = k;
      *cmax_off = off;
    }
  }
  return sw;
}

/* X-drop (wavefront/wavefront_heuristic.c:326-380): cells whose score fell
 * xdrop or more below the best seen so far are cut from both ends. */
static void hs_xdrop(oracle_ua_t* ua, orow_t* m) {
  const pen_t* p = ua->p;
  if (ua->steps_wait > 0) return;
  int cmax, cmax_k;
  int32_t cmax_off;
  const int base = m->lo;
  int* sw = hs_sw_scores(ua, m, &cmax, &cmax_k, &cmax_off);
  if (ua->max_sw_k != INT32_MAX) {
    int k;
    for (k = m->lo; k <= m->hi; ++k) {
      if (m->off[k] < 0) continue;
      if (wsub(ua->max_sw, sw[k - base]) < p->h_xdrop) break;
    }
    m->lo = k;
    for (k = m->hi; k >= m->lo; --k) {
      if (m->off[k] < 0) continue;
      if (wsub(ua->max_sw, sw[k - base]) < p->h_xdrop) break;
    }
    m->hi = k;
    if (cmax > ua->max_sw) {
      ua->max_sw = cmax;
      ua->max_sw_k = cmax_k;
    }
  } else {
    ua->max_sw = cmax;
    ua->max_sw_k = cmax_k;
  }
  free(sw);
  ua->steps_wait = p->h_steps;
}

/* Z-drop (wavefront/wavefront_heuristic.c:397-450): ends the alignment once
 * the best score of a wavefront falls more than zdrop below the best seen,
 * at the position of that best.  Returns 1 when dropped. */
static int hs_zdrop(oracle_ua_t* ua, orow_t* m) {
  const pen_t* p = ua->p;
  if (ua->steps_wait > 0) return 0;
  int cmax, cmax_k;
  int32_t cmax_off;
  free(hs_sw_scores(ua, m, &cmax, &cmax_k, &cmax_off));
  if (ua->max_sw_k != INT32_MAX) {
    if (cmax > ua->max_sw) {
      ua->max_sw = cmax;
      ua->max_wf_score = ua->s;
      ua->max_sw_k = cmax_k;
      ua->max_sw_off = cmax_off;
    } else if (wsub(ua->max_sw, cmax) > p->h_zdrop) {
      ua->zdropped = 1;
      ua->end_k = ua->max_sw_k;
      ua->end_off = ua->max_sw_off;
      return 1;
    }
  } else {
    ua->max_sw = cmax;
    ua->max_wf_score = ua->s;
    ua->max_sw_k = cmax_k;
    ua->max_sw_off = cmax_off;
  }
  ua->steps_wait = p->h_steps;
  return 0;
}

/* Banded, adaptive (wavefront/wavefront_heuristic.c:460-505): a band of
 * max_k-min_k+1 diagonals placed by sampling four cells' distances. */
static void hs_banded_adaptive(oracle_ua_t* ua, orow_t* m) {
  const pen_t* p = ua->p;
  if (ua->steps_wait > 0) return;
  const int lo = m->lo, hi = m->hi;
  const int len = hi - lo + 1;
  if (len < 4) return;
  const int max_len = p->h_max_k - p->h_min_k + 1;
  if (len > max_len) {
    const int leeway = (len - max_len) / 2;
    const int quarter = len / 4;
    const int d0 = hs_distance(ua, lo, m->off[lo], 0);
    const int d1 = hs_distance(ua, lo + quarter, m->off[lo + quarter], 0);
    const int d2 = hs_distance(ua, lo + 2 * quarter, m->off[lo + 2 * quarter], 0);
    const int d3 = hs_distance(ua, hi, m->off[hi], 0);
    int nlo = lo;
    if (d0 > d3) nlo += leeway;
    if (d1 > d2) nlo += leeway;
    m->lo = imax(nlo, lo);
    m->hi = imin(nlo + max_len - 1, hi);
  }
  ua->steps_wait = p->h_steps;
}

/* Heuristic cut-off of the extended M[s] (dispatcher,
 * wavefront/wavefront_heuristic.c:506-563).  Only the limits shrink: the cut
 * offsets stay inside the initialised window, where later compute steps
 * (wavefront/wavefront_compute.c:498-527 pads only beyond it) and the
 * back-trace (wavefront/wavefront_backtrace.c:63-75) still read them.  I/D
 * rows of the same score take the intersection of limits.  Returns 1 when
 * z-drop ends the alignment. */
static int heuristic_cutoff(oracle_ua_t* ua) {
  oracle_ws_t* ws = ua->ws;
  const pen_t* p = ua->p;
  orow_t* m = row_at(ws, ua->s, C_M);
  if (!m->exists || m->lo > m->hi) return 0;
  --ua->steps_wait;
  const int lo = m->lo, hi = m->hi;
  if (p->heur & HS_WFADAPTIVE) {
    hs_wfadaptive(ua, m, 0);
  } else if (p->heur & HS_WFMASH) {
    hs_wfadaptive(ua, m, 1);
  }
  if (p->heur & HS_XDROP) {
    hs_xdrop(ua, m);
  } else if (p->heur & HS_ZDROP) {
    if (hs_zdrop(ua, m)) return 1;
  }
  if (p->heur & HS_BANDED_STATIC) {
    if (m->lo < p->h_min_k) m->lo = p->h_min_k;
    if (m->hi > p->h_max_k) m->hi = p->h_max_k;
  } else if (p->heur & HS_BANDED_ADAPTIVE) {
    hs_banded_adaptive(ua, m);
  }
  if (m->lo == lo && m->hi == hi) return 0;
  if (m->lo > m->hi && !m->null) m->null = m->cut_null = 1;
  if (p->metric <= 2) return 0;
  const int ncomp = p->metric == 4 ? NCOMP : 3;
  for (int c = 1; c < ncomp; ++c) {
    orow_t* r = row_at(ws, ua->s, c);
    if (!r->exists) continue;
    if (m->lo > r->lo) r->lo = m->lo;
    if (m->hi < r->hi) r->hi = m->hi;
    if (r->lo > r->hi && !r->null) r->null = r->cut_null = 1;
  }
  return 0;
}

/* Extends M[s] and tests termination on component ce
 * (wavefront/wavefront_extend.c:86-121,173-212,
 * wavefront/wavefront_termination.c:37-114).  Returns ST_END_REACHED,
 * ST_END_UNREACHABLE or 0; *max_ak (if given) receives the largest
 * antidiagonal 2*offset-k of the extended cells, or 0
 * (wavefront/wavefront_extend_kernels.c:130-153). */
int oracle_ua_extend(oracle_ua_t* ua, int* max_ak) {
  oracle_ws_t* ws = ua->ws;
  if (max_ak) *max_ak = 0;
  orow_t* m = row_at(ws, ua->s, C_M);
  if (!m->exists) {
    /* (edit and indel with a step limit run on past null wavefronts, as
     * the reference's edit driver does: see align_one_impl) */
    if (ua->null_steps > ua->p->scope &&
        !(ua->p->metric <= 1 && ua->p->max_steps != INT_MAX))
      return ST_END_UNREACHABLE;
    return 0;
  }
  int mak = 0;
  for (int k = m->lo; k <= m->hi; ++k) {
    const int32_t off = m->off[k];
    if (off == WF_NULL) continue;
    const int L = lcp(ua->P, ua->plen, ua->T, ua->tlen, off - k, off);
    m->off[k] = off + L;
    ua->ext += L;
    const int ak = 2 * (off + L) - k;
    if (mak < ak) mak = ak;
    /* ends-free: the first diagonal, in extension order, that reaches the end
     * of one sequence with the other's rest within its end-free length
     * (wavefront/wavefront_extend_kernels.c:154-194,
     * wavefront/wavefront_termination.c:115-162) */
    if (ua->endsfree) {
      const int h = off + L, v = off + L - k;
      if ((h >= ua->tlen && ua->plen - v <= ua->pef) || (v >= ua->plen && ua->tlen - h <= ua->tef)) {
        ua->end_k = k;
        ua->end_off = off + L;
        return ST_END_REACHED;
      }
    }
  }
  if (ua->endsfree) {
    if (ua->heur && heuristic_cutoff(ua)) return ST_END_UNREACHABLE;
    if (max_ak) *max_ak = mak;
    return 0;
  }
  const orow_t* e = row_at(ws, ua->s, ua->ce);
  const int k_end = ua->k_end;
  if (e->exists && e->lo <= k_end && k_end <= e->hi && e->off[k_end] >= ua->tlen)
    return ST_END_REACHED;
  /* wavefront/wavefront_extend.c:112-119 */
  if (ua->heur && heuristic_cutoff(ua)) return ST_END_UNREACHABLE;
  if (max_ak) *max_ak = mak;
  return 0;
}

/* Computes wavefront s+1 (wavefront/wavefront_unialign.c:266-268). */
void oracle_ua_compute(oracle_ua_t* ua) {
  ua->s++;
  ua->cells += compute_step(ua->ws, ua->p, ua->s, ua->plen, ua->tlen, &ua->null_steps,
                            ua->endsfree);
}

/* Full back-trace of a finished stepper into ops (forward order); returns the
 * number of operations or -1. */
int oracle_ua_backtrace(oracle_ua_t* ua, char* ops) {
  /* the reference's CIGAR buffer holds 2*(plen+tlen) operations
   * (wavefront/wavefront_aligner.c:403-405); a trace through stale sources
   * can be longer than plen+tlen */
  const int cap = 2 * (ua->plen + ua->tlen) + 8;
  char* rev = (char*)malloc((size_t)cap);
  const int n = backtrace(ua->ws, ua->p, ua->plen, ua->tlen, ua->s, ua->end_k, ua->end_off, ua->ce,
                          rev, cap, &ua->stale_source);
  if (n >= 0)
    for (int i = 0; i < n; ++i) ops[i] = rev[n - 1 - i];
  free(rev);
  return n;
}

int oracle_classic_score(const pen_t* p, int plen, int tlen, int s) {
  return classic_score(p, plen, tlen, s);
}

/* Score of an operation run under the user's penalties, as maximal-score
 * trimming counts it (alignment/cigar_utils.c:112-318: a match earns -match,
 * or 1 when match is 0). */
static int run_score_affine2p(const pen_t* p, char op, int len, int* ev, int* eh) {
  switch (op) {
    case 'M': *ev += len; *eh += len; return (p->um != 0 ? p->um : -1) * len;
    case 'X': *ev += len; *eh += len; return p->ux * len;
    case 'D': {
      *ev += len;
      const int a = p->uo1 + p->ue1 * len, b = p->uo2 + p->ue2 * len;
      return a < b ? a : b;
    }
    default: {
      *eh += len;
      const int a = p->uo1 + p->ue1 * len, b = p->uo2 + p->ue2 * len;
      return a < b ? a : b;
    }
  }
}

/* Maximal-score trimming of ops[0..*n) (alignment/cigar_utils.c:112-318,
 * dispatch wavefront/wavefront_aligner.c:664-676).  On return *n, *score and
 * *ev/*eh describe the kept prefix (an empty prefix: *n = 0, score INT32_MIN,
 * end (-1,-1), as cigar_clear leaves them); returns 1 if the CIGAR was trimmed. */
static int maxtrim(const pen_t* p, const char* ops, int* n, int* score, int* ev, int* eh) {
  const int len = *n;
  int max_score = 0, max_off = 0, max_v = 0, max_h = 0;
  int sc = 0, v = 0, h = 0;
  if (p->metric == 2) {
    /* cigar_maxtrim_gap_linear (alignment/cigar_utils.c:112-160) */
    const int mscore = p->um != 0 ? p->um : -1;
    for (int i = 0; i < len; ++i) {
      switch (ops[i]) {
        case 'M': sc -= mscore; ++v; ++h; break;
        case 'X': sc -= p->ux; ++v; ++h; break;
        case 'I': sc -= p->uo1; ++h; break;
        default: sc -= p->uo1; ++v; break;
      }
      if (max_score < sc) {
        max_score = sc;
        max_off = i;
        max_v = v;
        max_h = h;
      }
    }
  } else if (p->metric == 4) {
    if (len <= 0) return 0;
    char last = 0;
    int run = 0;
    for (int i = 0; i < len; ++i) {
      if (ops[i] != last && last != 0) {
        sc -= run_score_affine2p(p, last, run, &v, &h);
        run = 0;
        if (max_score < sc) {
          max_score = sc;
          max_off = i - 1;
          max_v = v;
          max_h = h;
        }
      }
      last = ops[i];
      ++run;
    }
    sc -= run_score_affine2p(p, last, run, &v, &h);
    if (max_score < sc) {
      max_score = sc;
      max_off = len - 1;
      max_v = v;
      max_h = h;
    }
  } else {
    const int mscore = p->um != 0 ? p->um : -1;
    char last = 0;
    for (int i = 0; i < len; ++i) {
      switch (ops[i]) {
        case 'M': sc -= mscore; ++v; ++h; break;
        case 'X': sc -= p->ux; ++v; ++h; break;
        case 'I': sc -= p->ue1 + (last == 'I' ? 0 : p->uo1); ++h; break;
        default: sc -= p->ue1 + (last == 'D' ? 0 : p->uo1); ++v; break;
      }
      last = ops[i];
      if (max_score < sc) {
        max_score = sc;
        max_off = i;
        max_v = v;
        max_h = h;
      }
    }
  }
  const int trimmed = (max_off != len - 1);
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

/* Wavefronts the reference allocates for a pair in high-memory mode
 * (wavefront/wavefront_components.c:41-124). */
static int64_t score_table_size(const pen_t* p, int plen, int tlen) {
  const int64_t mn = imin(plen, tlen), diff = plen > tlen ? plen - tlen : tlen - plen;
  if (p->metric <= 1) return imax(plen, tlen) + 1;
  if (p->metric == 2) return mn * p->x + (int64_t)p->o1 * diff + 1;
  int64_t indel = p->o1 + diff * p->e1;
  if (p->metric == 4) {
    const int64_t indel2 = p->o2 + diff * p->e2;
    if (indel2 < indel) indel = indel2;
  }
  return mn * p->x + indel + 1;
}

/* One unidirectional alignment (wavefront/wavefront_unialign.c:242-273),
 * writing up to 2*(plen+tlen)+8 operations into ops. */
static void align_one_impl(oracle_ws_t* ws, const pen_t* p, const char* P, int plen,
                           const char* T, int tlen, int32_t* out_score, int32_t* out_status,
                           char* ops, int32_t* ops_len, int64_t* cells, int64_t* ext,
                           int32_t* end, int32_t* flags) {
  int32_t end_dummy[2];
  if (!end) end = end_dummy;
  end[0] = end[1] = -1;
  oracle_ua_t ua;
  if (p->endsfree) {
    /* extension presets (wavefront/wavefront_align.c:57-63), then the bounds
     * check of :90-101 (the reference exits there) */
    const int pbf = p->extension ? 0 : p->pbf, pef = p->extension ? plen : p->pef;
    const int tbf = p->extension ? 0 : p->tbf, tef = p->extension ? tlen : p->tef;
    if (pbf > plen || pef > plen || tbf > tlen || tef > tlen) {
      if (cells) *cells = 0;
      if (ext) *ext = 0;
      *out_score = 0;
      *out_status = ST_INVALID_FORM;
      *ops_len = 0;
      return;
    }
    oracle_ua_start_endsfree(&ua, ws, p, P, plen, T, tlen, pbf, pef, tbf, tef);
  } else {
    oracle_ua_start(&ua, ws, p, P, plen, T, tlen, C_M, C_M);
  }
  int status;
  while (1) {
    status = oracle_ua_extend(&ua, NULL);
    if (status) break;
    oracle_ua_compute(&ua);
    /* Edit and indel: a null wavefront does not end the reference's
     * alignment.  Its extend step counts null steps only for a missing
     * wavefront (wavefront/wavefront_extend.c:93-101), and the edit driver
     * allocates every one (wavefront/wavefront_compute_edit.c:321-374).  No
     * later cell can be valid, so only the step limit ends it.  Without a
     * step limit the reference never ends; the checker ends it as
     * unreachable instead. */
    if (p->metric <= 1 && ua.null_steps >= INT_MAX / 2 && p->max_steps != INT_MAX)
      ua.s = p->max_steps;
    /* wavefront/wavefront_unialign.c:102-107 */
    if (ua.s >= p->max_steps) {
      /* the reference exits before the step limit once the score passes its
       * wavefront table (wavefront/wavefront_compute.c:442-446) */
      if (!p->score_only && ua.s >= score_table_size(p, plen, tlen))
        *flags |= ORACLE_FLAG_OVER_BOUND;
      if (ext) *ext = ua.ext;
      if (cells) *cells = ua.cells;
      *out_score = -p->max_steps;
      *out_status = ST_MAX_STEPS;
      *ops_len = 0;
      return;
    }
  }
  if (cells) *cells = ua.cells;
  if (ext) *ext = ua.ext;
  /* a heuristic can run an alignment past the score bound the reference
   * sizes its wavefront table by (wavefront/wavefront_components.c:41-124);
   * it exits there (wavefront/wavefront_compute.c:442-446) unless an earlier,
   * longer pair of the same aligner grew the table */
  if (!p->score_only && ua.s >= score_table_size(p, plen, tlen)) *flags |= ORACLE_FLAG_OVER_BOUND;
  if (status == ST_END_UNREACHABLE) {
    /* wavefront/wavefront_unialign.c:147-237.  The end position is z-drop's
     * best cell, or none (DPMATRIX_DIAGONAL_NULL, WAVEFRONT_OFFSET_NULL) when
     * the null steps ran out. */
    const int k = ua.zdropped ? ua.end_k : INT32_MAX;
    const int32_t off = ua.zdropped ? ua.end_off : WF_NULL;
    *out_status = 1; /* WF_STATUS_ALG_PARTIAL */
    if (p->score_only || ops == NULL) {
      end[0] = wsub(off, k);
      end[1] = off;
      *out_score = classic_score_wrapped(p, end[0], end[1], ua.s);
      *ops_len = 0;
      return;
    }
    /* the back-trace starts from the current score at that cell, adding the
     * gaps to both ends (wavefront/wavefront_backtrace.c:339-356); then the
     * maximal-score trim (wavefront/wavefront_aligner.c:664-676) */
    int n = 0, sc = INT32_MIN, ev = -1, eh = -1;
    if (ua.zdropped) {
      n = oracle_ua_backtrace(&ua, ops);
      if (ua.stale_source) *flags |= ORACLE_FLAG_STALE_SOURCE;
      if (n < 0) {
        *out_status = ST_UNATTAINABLE;
        *ops_len = 0;
        *out_score = 0;
        return;
      }
      sc = ua.s;
    }
    if (p->metric > 1 && !(p->metric == 4 && n == 0)) maxtrim(p, ops, &n, &sc, &ev, &eh);
    *ops_len = n;
    *out_score = sc;
    end[0] = ev;
    end[1] = eh;
    return;
  }
  /* wavefront/wavefront_unialign.c:147-237 */
  *out_score = classic_score(p, plen, tlen, ua.s);
  *out_status = ST_COMPLETED;
  if (p->score_only || ops == NULL) {
    end[0] = plen;
    end[1] = tlen;
    *ops_len = 0;
    return;
  }
  int n = oracle_ua_backtrace(&ua, ops);
  if (ua.stale_source) *flags |= ORACLE_FLAG_STALE_SOURCE;
  if (n < 0) {
    *out_status = ST_UNATTAINABLE;
    *ops_len = 0;
    end[0] = end[1] = -1;
    return;
  }
  *ops_len = n;
  if (p->extension) {
    int sc = 0, ev = 0, eh = 0;
    if (p->metric <= 1 || (p->metric == 4 && *ops_len == 0)) {
      /* no trimming for edit and indel (wavefront/wavefront_aligner.c:
       * 664-676), nor of an empty affine2p CIGAR (alignment/cigar_utils.c:281):
       * the CIGAR stays as the back-trace wrote it, with the WFA score and no
       * end position */
      *out_status = ST_COMPLETED;
      *out_score = ua.s;
      return;
    }
    *out_status = maxtrim(p, ops, &n, &sc, &ev, &eh) ? 1 /* WF_STATUS_ALG_PARTIAL */ : ST_COMPLETED;
    *ops_len = n;
    *out_score = sc;
    end[0] = ev;
    end[1] = eh;
    return;
  }
  end[0] = ua.end_off - ua.end_k;
  end[1] = ua.end_off;
  if (ua.endsfree) *out_score = classic_score(p, end[0], end[1], ua.s);
}

/* The same with the caller's buffer of plen+tlen operations.  flags (if
 * given) receives ORACLE_FLAG_* bits; a CIGAR longer than the buffer (a trace
 * through stale sources) is reported with ops_len = -1. */
void oracle_align_one(oracle_ws_t* ws, const pen_t* p, const char* P, int plen, const char* T,
                      int tlen, int32_t* out_score, int32_t* out_status, char* ops,
                      int32_t* ops_len, int64_t* cells, int64_t* ext, int32_t* end,
                      int32_t* flags) {
  char* full = ops ? (char*)malloc((size_t)(2 * (plen + tlen) + 8)) : NULL;
  int32_t fl = 0;
  align_one_impl(ws, p, P, plen, T, tlen, out_score, out_status, full, ops_len, cells, ext, end,
                 &fl);
  if (ops) {
    if (*ops_len > plen + tlen) {
      *ops_len = -1;
    } else if (*ops_len > 0) {
      memcpy(ops, full, (size_t)*ops_len);
    }
    free(full);
  }
  if (flags) *flags = fl;
}

int oracle_align_batch(const int* cfg, int num_pairs, const char* sequences, const int64_t* p_off,
                       const int32_t* p_len, const int64_t* t_off, const int32_t* t_len,
                       int32_t* out_score, int32_t* out_status, char* out_ops,
                       const int64_t* ops_off, int32_t* out_ops_len, int64_t* out_cells,
                       int64_t* out_ext, int32_t* out_end, int nthreads) {
  return oracle_align_batch_flags(cfg, num_pairs, sequences, p_off, p_len, t_off, t_len,
                                  out_score, out_status, out_ops, ops_off, out_ops_len, out_cells,
                                  out_ext, out_end, NULL, nthreads);
}

int oracle_align_batch_flags(const int* cfg, int num_pairs, const char* sequences,
                             const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                             const int32_t* t_len, int32_t* out_score, int32_t* out_status,
                             char* out_ops, const int64_t* ops_off, int32_t* out_ops_len,
                             int64_t* out_cells, int64_t* out_ext, int32_t* out_end,
                             int32_t* out_flags, int nthreads) {
  pen_t p;
  if (setup_penalties(cfg, &p) != 0) return -1;
  const int ultralow = (cfg[7] == 3);
  /* BiWFA has no ends-free or extension form (wavefront/wavefront_align.c:67-82) */
  if (ultralow && p.endsfree) return -1;
  /* BiWFA is restated with every heuristic but z-drop (whose drop inside a
   * breakpoint search is not restated) */
  if (ultralow && (p.heur & HS_ZDROP)) return -1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    oracle_ws_t ws;
    oracle_ws_init(&ws, p.score_only && !ultralow, p.scope);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < num_pairs; ++i) {
      char* ops = (out_ops && !p.score_only) ? out_ops + ops_off[i] : NULL;
      int64_t* cells = out_cells ? &out_cells[i] : NULL;
      int64_t* ext = out_ext ? &out_ext[i] : NULL;
      int32_t* end = out_end ? &out_end[2 * i] : NULL;
      if (ultralow) {
        oracle_bialign(&p, sequences + p_off[i], p_len[i], sequences + t_off[i], t_len[i], &ws,
                       &out_score[i], &out_status[i], ops, &out_ops_len[i], cells, ext, end);
      } else {
        oracle_align_one(&ws, &p, sequences + p_off[i], p_len[i], sequences + t_off[i], t_len[i],
                         &out_score[i], &out_status[i], ops, &out_ops_len[i], cells, ext, end,
                         out_flags ? &out_flags[i] : NULL);
      }
    }
    ws_free(&ws);
  }
  return 0;
}


/*
 * wfa_datagen.c -- seeded synthetic pair generator (the role of the
 * reference's tools/generate_dataset, which is unseeded:
 * tools/generate_dataset/generate_dataset.c:366).
 *
 * Every pair is a pure function of (workload, pair index): a SplitMix64
 * stream seeded with (workload << 40) ^ pair, so any sub-range of a workload
 * can be regenerated on any host (x86 or Arm) with identical bytes.
 *
 * Workloads (pattern: i.i.d. uniform ACGT; text: the pattern with edits
 * applied one after another at uniform positions of the current text; a
 * mismatch always changes the base, as tools/generate_dataset/generate_dataset.c:151-154):
 *   0  |P|=100; exactly 5 edits; each mismatch / 1-bp insertion / 1-bp deletion w.p. 1/3
 *   1  |P|~U[500,1500]; d~U[0,0.15]; round(d|P|) edits as in 0, except that
 *      10% of insertions/deletions have length Geometric(0.5) (>=1)
 *   2  |P| log-uniform in [1000,10000]; d=0.05; 20% of edits are insertions or
 *      deletions of length U[20,200], the rest as in 0
 *   3  |P|=100000; d~U[0.10,0.15]; 50% mismatches, 50% insertions/deletions of
 *      length Geometric(0.3)
 *   4  |P| lognormal (median 2000, sigma 1.0; the normal is drawn as a sum of
 *      12 uniforms) clipped to [100,50000];
 *      d~U[0.01,0.20]; edits as in 0
 *   5  |P| given by `param` (fixed); d given by `param2/1000`; edits as in 0
 *   6  as 5, then |P|/2 random bases appended to the text (very different lengths)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  uint64_t s;
} rng_t;

static uint64_t rng_next(rng_t* r) {
  uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double rng_u01(rng_t* r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static uint32_t rng_below(rng_t* r, uint32_t n) {
  return (uint32_t)(((rng_next(r) >> 32) * (uint64_t)n) >> 32);
}
static int rng_geometric(rng_t* r, double p) { /* support >= 1 */
  int k = 1;
  while (rng_u01(r) >= p && k < 1000000) ++k;
  return k;
}
/* Approximate standard normal (Irwin-Hall, 12 uniforms): only +/- so the
 * result is bit-identical on every IEEE host. */
static double rng_normal(rng_t* r) {
  double s = 0.0;
  for (int i = 0; i < 12; ++i) s += rng_u01(r);
  return s - 6.0;
}
/* exp() from basic IEEE operations only (range reduction + Taylor series);
 * compiled with -ffp-contract=off it is bit-identical across hosts. */
static double det_exp(double x) {
  const double ln2 = 0.6931471805599453;
  const double n = floor(x / ln2 + 0.5);
  const double rr = x - n * ln2;
  double term = 1.0, sum = 1.0;
  for (int i = 1; i < 20; ++i) {
    term = term * rr / (double)i;
    sum += term;
  }
  return ldexp(sum, (int)n);
}

static const char kBases[4] = {'A', 'C', 'G', 'T'};

typedef struct {
  char* buf;
  int len, cap;
} text_t;

static void text_reserve(text_t* t, int n) {
  if (n <= t->cap) return;
  int c = t->cap ? t->cap : 256;
  while (c < n) c *= 2;
  t->buf = (char*)realloc(t->buf, (size_t)c);
  t->cap = c;
}

/* Generates pair `pair` of `workload` into P (pattern) and T (text). */
static void gen_pair(int workload, int64_t pair, int param, int param2, text_t* P, text_t* T) {
  rng_t r;
  r.s = ((uint64_t)workload << 40) ^ (uint64_t)pair;
  rng_next(&r);
  int plen;
  double d = 0.0;
  int fixed_edits = -1;
  switch (workload) {
    case 0: plen = 100; fixed_edits = 5; break;
    case 1: plen = 500 + (int)rng_below(&r, 1001); d = 0.15 * rng_u01(&r); break;
    case 2: plen = (int)floor(1000.0 * det_exp(2.302585092994046 * rng_u01(&r))); d = 0.05; break;
    case 3: plen = 100000; d = 0.10 + 0.05 * rng_u01(&r); break;
    case 4: {
      double l = 2000.0 * det_exp(1.0 * rng_normal(&r));
      if (l < 100) l = 100;
      if (l > 50000) l = 50000;
      plen = (int)l;
      d = 0.01 + 0.19 * rng_u01(&r);
      break;
    }
    default: plen = param > 0 ? param : 1000; d = param2 / 1000.0; break;
  }
  text_reserve(P, plen + 1);
  for (int i = 0; i < plen; ++i) P->buf[i] = kBases[rng_below(&r, 4)];
  P->len = plen;
  const int nedits = fixed_edits >= 0 ? fixed_edits : (int)floor(d * plen + 0.5);
  text_reserve(T, plen + 1);
  memcpy(T->buf, P->buf, (size_t)plen);
  T->len = plen;
  for (int e = 0; e < nedits; ++e) {
    int type; /* 0 mismatch, 1 insertion, 2 deletion */
    int len = 1;
    if (workload == 3) {
      if (rng_below(&r, 2) == 0) type = 0;
      else { type = 1 + (int)rng_below(&r, 2); len = rng_geometric(&r, 0.3); }
    } else if (workload == 2 && rng_u01(&r) < 0.2) {
      type = 1 + (int)rng_below(&r, 2);
      len = 20 + (int)rng_below(&r, 181);
    } else {
      type = (int)rng_below(&r, 3);
      if (workload == 1 && type != 0 && rng_u01(&r) < 0.1) len = rng_geometric(&r, 0.5);
    }
    if (type == 0) {
      if (T->len == 0) continue;
      const int pos = (int)rng_below(&r, (uint32_t)T->len);
      const char old = T->buf[pos];
      int idx = 0;
      while (kBases[idx] != old) ++idx;
      T->buf[pos] = kBases[(idx + 1 + rng_below(&r, 3)) & 3];
    } else if (type == 1) {
      const int pos = (int)rng_below(&r, (uint32_t)T->len + 1);
      text_reserve(T, T->len + len + 1);
      memmove(T->buf + pos + len, T->buf + pos, (size_t)(T->len - pos));
      for (int i = 0; i < len; ++i) T->buf[pos + i] = kBases[rng_below(&r, 4)];
      T->len += len;
    } else {
      if (T->len == 0) continue;
      const int pos = (int)rng_below(&r, (uint32_t)T->len);
      if (len > T->len - pos) len = T->len - pos;
      memmove(T->buf + pos, T->buf + pos + len, (size_t)(T->len - pos - len));
      T->len -= len;
    }
  }
  if (workload == 6) {
    /* workload 5 with a random tail of half the pattern's length appended to
     * the text: pairs of very different lengths */
    const int tail = plen / 2;
    text_reserve(T, T->len + tail + 1);
    for (int i = 0; i < tail; ++i) T->buf[T->len + i] = kBases[rng_below(&r, 4)];
    T->len += tail;
  }
}

/* Lengths of pairs [first, first+n) of a workload. */
void wf2g_generate_lengths(int workload, int64_t first, int n, int param, int param2,
                           int32_t* p_len, int32_t* t_len) {
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    text_t P = {0}, T = {0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
    for (int i = 0; i < n; ++i) {
      gen_pair(workload, first + i, param, param2, &P, &T);
      p_len[i] = P.len;
      t_len[i] = T.len;
    }
    free(P.buf);
    free(T.buf);
  }
}

/* Writes pairs [first, first+n) into seqs: pattern i at p_off[i], text i at
 * t_off[i] (offsets are chosen by the caller, typically from the lengths
 * returned by wf2g_generate_lengths). */
void wf2g_generate_pairs(int workload, int64_t first, int n, int param, int param2, char* seqs,
                         const int64_t* p_off, const int64_t* t_off) {
#ifdef _OPENMP
#pragma omp parallel
#endif
  {
    text_t P = {0}, T = {0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
    for (int i = 0; i < n; ++i) {
      gen_pair(workload, first + i, param, param2, &P, &T);
      memcpy(seqs + p_off[i], P.buf, (size_t)P.len);
      memcpy(seqs + t_off[i], T.buf, (size_t)T.len);
    }
    free(P.buf);
    free(T.buf);
  }
}

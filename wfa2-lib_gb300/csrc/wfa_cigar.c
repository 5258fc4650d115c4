/*
 * wfa_cigar.c -- the cigar_t helpers of the drop-in API (host C).
 *
 * Same contract as the reference's alignment/cigar.c: the operations
 * 'M','X','I','D' live in operations[begin_offset, end_offset); the SAM CIGAR
 * is derived lazily; scores follow the penalty conventions of
 * alignment/cigar.c:245-346 (score = -penalty, match <= 0 adds).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wfa2gpu.h"

/* SAM operation codes (SAM v1 spec) */
enum { SAM_M = 0, SAM_I = 1, SAM_D = 2, SAM_N = 3, SAM_EQ = 7, SAM_X = 8, SAM_NA = 15 };

static uint32_t sam_code(char op) {
  switch (op) {
    case 'M': return SAM_M;
    case 'I': return SAM_I;
    case 'D': return SAM_D;
    case 'N': return SAM_N;
    case '=': return SAM_EQ;
    case 'X': return SAM_X;
    default: return SAM_NA;
  }
}

cigar_t* cigar_new(const int max_operations) {
  cigar_t* c = (cigar_t*)malloc(sizeof(cigar_t));
  c->max_operations = max_operations;
  c->operations = (char*)malloc((size_t)max_operations);
  c->cigar_buffer = (uint32_t*)calloc((size_t)max_operations, sizeof(uint32_t));
  c->has_misms = false;
  cigar_clear(c);
  return c;
}
void cigar_clear(cigar_t* const c) {
  c->begin_offset = 0;
  c->end_offset = 0;
  c->score = INT32_MIN;
  c->end_v = -1;
  c->end_h = -1;
  c->cigar_length = 0;
}
void cigar_resize(cigar_t* const c, const int max_operations) {
  if (max_operations > c->max_operations) {
    free(c->operations);
    free(c->cigar_buffer);
    c->max_operations = max_operations;
    c->operations = (char*)malloc((size_t)max_operations);
    c->cigar_buffer = (uint32_t*)calloc((size_t)max_operations, sizeof(uint32_t));
  }
  cigar_clear(c);
}
void cigar_free(cigar_t* const c) {
  if (!c) return;
  free(c->operations);
  free(c->cigar_buffer);
  free(c);
}
bool cigar_is_null(const cigar_t* const c) { return c->begin_offset >= c->end_offset; }
int cigar_count_matches(const cigar_t* const c) {
  int n = 0;
  for (int i = c->begin_offset; i < c->end_offset; ++i) n += (c->operations[i] == 'M');
  return n;
}

void cigar_get_CIGAR(cigar_t* const c, const bool show_mismatches, uint32_t** const cigar_buffer,
                     int* const cigar_length) {
  if (c->cigar_length == 0 || c->has_misms != show_mismatches) {
    int n = 0;
    if (c->begin_offset < c->end_offset) {
      char last = c->operations[c->begin_offset];
      if (!show_mismatches && last == 'X') last = 'M';
      uint32_t run = 1;
      for (int i = c->begin_offset + 1; i <= c->end_offset; ++i) {
        char op = (i < c->end_offset) ? c->operations[i] : '\0';
        if (!show_mismatches && op == 'X') op = 'M';
        if (i < c->end_offset && op == last) {
          ++run;
          continue;
        }
        const uint32_t code = (show_mismatches && last == 'M') ? SAM_EQ : sam_code(last);
        c->cigar_buffer[n++] = (run << 4) | code;
        last = op;
        run = 1;
      }
    }
    c->has_misms = show_mismatches;
    c->cigar_length = n;
  }
  *cigar_buffer = c->cigar_buffer;
  *cigar_length = c->cigar_length;
}

static void unknown_op(void) {
  fprintf(stderr, "[CIGAR] Computing CIGAR score: Unknown operation\n");
  exit(1);
}
int cigar_score_edit(const cigar_t* const c) {
  int s = 0;
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    const char op = c->operations[i];
    if (op == 'X' || op == 'I' || op == 'D') ++s;
    else if (op != 'M') unknown_op();
  }
  return s;
}
int cigar_score_gap_linear(const cigar_t* const c, const linear_penalties_t* const p) {
  int s = 0;
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    switch (c->operations[i]) {
      case 'M': s -= p->match; break;
      case 'X': s -= p->mismatch; break;
      case 'I':
      case 'D': s -= p->indel; break;
      default: unknown_op();
    }
  }
  return s;
}
int cigar_score_gap_affine(const cigar_t* const c, const affine_penalties_t* const p) {
  int s = 0;
  char last = '\0';
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    const char op = c->operations[i];
    switch (op) {
      case 'M': s -= p->match; break;
      case 'X': s -= p->mismatch; break;
      case 'I':
      case 'D': s -= p->gap_extension + (last == op ? 0 : p->gap_opening); break;
      default: unknown_op();
    }
    last = op;
  }
  return s;
}
static int affine2p_run(char op, int len, const affine2p_penalties_t* p) {
  switch (op) {
    case 'M': return p->match * len;
    case 'X': return p->mismatch * len;
    case 'I':
    case 'D': {
      const int a = p->gap_opening1 + p->gap_extension1 * len;
      const int b = p->gap_opening2 + p->gap_extension2 * len;
      return a < b ? a : b;
    }
    default: unknown_op();
  }
  return 0;
}
int cigar_score_gap_affine2p(const cigar_t* const c, const affine2p_penalties_t* const p) {
  int s = 0, run = 0;
  char last = '\0';
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    const char op = c->operations[i];
    if (op != last && last != '\0') {
      s -= affine2p_run(last, run, p);
      run = 0;
    }
    last = op;
    ++run;
  }
  s -= affine2p_run(last, run, p);
  return s;
}

/* Maximal-score trimming (alignment/cigar_utils.c:112-318): the CIGAR is cut
 * to its highest-scoring prefix under the penalties, where a match earns
 * -match (1 when match is 0).  A best prefix of score 0 clears the CIGAR;
 * otherwise its score and end position are set.  Returns whether the best
 * prefix ends before the last operation.  The affine2p rule scores whole
 * runs (each gap run the cheaper of its two models) and may end only at a
 * run's end. */
typedef struct {
  int score, v, h;
} trim_walk_t;
static bool maxtrim_apply(cigar_t* const c, int best, int best_i, int bv, int bh) {
  const bool trimmed = best_i != c->end_offset - 1;
  if (best == 0) {
    cigar_clear(c);
  } else {
    c->end_offset = best_i + 1;
    if (c->end_offset < c->max_operations) c->operations[c->end_offset] = '\0';
    c->score = best;
    c->end_v = bv;
    c->end_h = bh;
  }
  return trimmed;
}
static void trim_step(trim_walk_t* w, char op, int cost) {
  w->score -= cost;
  if (op == 'M' || op == 'X') {
    ++w->v;
    ++w->h;
  } else if (op == 'I') {
    ++w->h;
  } else {
    ++w->v;
  }
}
bool cigar_maxtrim_gap_linear(cigar_t* const c, const linear_penalties_t* const p) {
  const int earn = p->match != 0 ? p->match : -1;
  trim_walk_t w = {0, 0, 0};
  int best = 0, best_i = c->begin_offset, bv = 0, bh = 0;
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    const char op = c->operations[i];
    trim_step(&w, op, op == 'M' ? earn : op == 'X' ? p->mismatch : p->indel);
    if (w.score > best) {
      best = w.score;
      best_i = i;
      bv = w.v;
      bh = w.h;
    }
  }
  return maxtrim_apply(c, best, best_i, bv, bh);
}
bool cigar_maxtrim_gap_affine(cigar_t* const c, const affine_penalties_t* const p) {
  const int earn = p->match != 0 ? p->match : -1;
  trim_walk_t w = {0, 0, 0};
  int best = 0, best_i = c->begin_offset, bv = 0, bh = 0;
  char last = '\0';
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    const char op = c->operations[i];
    const int cost = op == 'M'   ? earn
                     : op == 'X' ? p->mismatch
                                 : p->gap_extension + (last == op ? 0 : p->gap_opening);
    trim_step(&w, op, cost);
    last = op;
    if (w.score > best) {
      best = w.score;
      best_i = i;
      bv = w.v;
      bh = w.h;
    }
  }
  return maxtrim_apply(c, best, best_i, bv, bh);
}
static int trim_run_2p(char op, int len, const affine2p_penalties_t* p, int* v, int* h) {
  if (op == 'M' || op == 'X') {
    *v += len;
    *h += len;
    return (op == 'M' ? (p->match != 0 ? p->match : -1) : p->mismatch) * len;
  }
  if (op == 'I') *h += len;
  else *v += len;
  const int a = p->gap_opening1 + p->gap_extension1 * len;
  const int b = p->gap_opening2 + p->gap_extension2 * len;
  return a < b ? a : b;
}
bool cigar_maxtrim_gap_affine2p(cigar_t* const c, const affine2p_penalties_t* const p) {
  if (c->begin_offset >= c->end_offset) return false;
  int score = 0, v = 0, h = 0, run = 0;
  int best = 0, best_i = c->begin_offset, bv = 0, bh = 0;
  char last = '\0';
  for (int i = c->begin_offset; i <= c->end_offset; ++i) {
    const char op = i < c->end_offset ? c->operations[i] : '\0';
    if (op != last && last != '\0') {  /* a run ends at i - 1 */
      score -= trim_run_2p(last, run, p, &v, &h);
      run = 0;
      if (score > best) {
        best = score;
        best_i = i - 1;
        bv = v;
        bh = h;
      }
    }
    last = op;
    ++run;
  }
  return maxtrim_apply(c, best, best_i, bv, bh);
}

bool cigar_check_alignment(FILE* const stream, const char* const pattern,
                           const int pattern_length, const char* const text,
                           const int text_length, const cigar_t* const c, const bool verbose) {
  int v = 0, h = 0;
  for (int i = c->begin_offset; i < c->end_offset; ++i) {
    switch (c->operations[i]) {
      case 'M':
        if (pattern[v] != text[h]) {
          if (verbose)
            fprintf(stream, "[CIGAR] Alignment not matching (pattern[%d]=%c != text[%d]=%c)\n", v,
                    pattern[v], h, text[h]);
          return false;
        }
        ++v;
        ++h;
        break;
      case 'X':
        if (pattern[v] == text[h]) {
          if (verbose)
            fprintf(stream, "[CIGAR] Alignment not mismatching (pattern[%d]=%c == text[%d]=%c)\n",
                    v, pattern[v], h, text[h]);
          return false;
        }
        ++v;
        ++h;
        break;
      case 'I': ++h; break;
      case 'D': ++v; break;
      default:
        fprintf(stream, "[CIGAR] Unknown edit operation '%c'\n", c->operations[i]);
        exit(1);
    }
  }
  if (v != pattern_length) {
    if (verbose)
      fprintf(stream, "[CIGAR] Alignment incorrect length (pattern-aligned=%d,pattern-length=%d)\n",
              v, pattern_length);
    return false;
  }
  if (h != text_length) {
    if (verbose)
      fprintf(stream, "[CIGAR] Alignment incorrect length (text-aligned=%d,text-length=%d)\n", h,
              text_length);
    return false;
  }
  return true;
}

int cigar_sprint(char* const buffer, const cigar_t* const c, const bool print_matches) {
  if (cigar_is_null(c)) {
    buffer[0] = '\0';
    return 0;
  }
  int cur = 0;
  char last = c->operations[c->begin_offset];
  int run = 1;
  for (int i = c->begin_offset + 1; i <= c->end_offset; ++i) {
    if (i < c->end_offset && c->operations[i] == last) {
      ++run;
      continue;
    }
    if (print_matches || last != 'M') cur += sprintf(buffer + cur, "%d%c", run, last);
    if (i < c->end_offset) last = c->operations[i];
    run = 1;
  }
  buffer[cur] = '\0';
  return cur;
}
void cigar_print(FILE* const stream, const cigar_t* const c, const bool print_matches) {
  if (cigar_is_null(c)) return;
  char* buf = (char*)malloc(2 * (size_t)(c->end_offset - c->begin_offset) + 20);
  cigar_sprint(buf, c, print_matches);
  fputs(buf, stream);
  free(buf);
}
int cigar_sprint_SAM_CIGAR(char* const buffer, cigar_t* const c, const bool show_mismatches) {
  uint32_t* ops;
  int n;
  cigar_get_CIGAR(c, show_mismatches, &ops, &n);
  int cur = 0;
  for (int i = 0; i < n; ++i) {
    const uint32_t code = ops[i] & 0xf;
    const char ch = code <= 8 ? "MIDN---=X"[code] : '?';
    cur += sprintf(buffer + cur, "%u%c", ops[i] >> 4, ch);
  }
  buffer[cur] = '\0';
  return cur;
}
void cigar_print_SAM_CIGAR(FILE* const stream, cigar_t* const c, const bool show_mismatches) {
  if (cigar_is_null(c)) return;
  char* buf = (char*)malloc(4 * (size_t)(c->end_offset - c->begin_offset) + 20);
  cigar_sprint_SAM_CIGAR(buf, c, show_mismatches);
  fputs(buf, stream);
  free(buf);
}
/* Three-line view: pattern, match markers, text (gaps as '-'). */
void cigar_print_pretty(FILE* const stream, cigar_t* const c, const char* const pattern,
                        const int pattern_length, const char* const text,
                        const int text_length) {
  (void)pattern_length;
  (void)text_length;
  const int n = c->end_offset - c->begin_offset;
  if (n <= 0) return;
  char* a = (char*)malloc((size_t)n + 1);
  char* m = (char*)malloc((size_t)n + 1);
  char* b = (char*)malloc((size_t)n + 1);
  int v = 0, h = 0;
  for (int i = 0; i < n; ++i) {
    const char op = c->operations[c->begin_offset + i];
    if (op == 'M' || op == 'X') {
      a[i] = pattern[v++];
      b[i] = text[h++];
      m[i] = (op == 'M') ? '|' : ' ';
    } else if (op == 'I') {
      a[i] = '-';
      b[i] = text[h++];
      m[i] = ' ';
    } else {
      a[i] = pattern[v++];
      b[i] = '-';
      m[i] = ' ';
    }
  }
  a[n] = m[n] = b[n] = '\0';
  fprintf(stream, "      ALIGNMENT ");
  cigar_print(stream, c, true);
  fprintf(stream, "\n      PATTERN    %s\n                 %s\n      TEXT       %s\n", a, m, b);
  free(a);
  free(m);
  free(b);
}

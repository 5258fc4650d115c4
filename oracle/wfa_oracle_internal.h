/*
 * wfa_oracle_internal.h -- types shared by the CPU restatement's translation
 * units (TEST INFRASTRUCTURE ONLY; see wfa_oracle.h).
 */
#ifndef WFA_ORACLE_INTERNAL_H_
#define WFA_ORACLE_INTERNAL_H_

#include <stddef.h>
#include <stdint.h>

/* wavefront/wavefront_offset.h:40-46 */
#define WF_NULL (INT32_MIN / 2)

/* wavefront/wfa.h:46-55 */
#define ST_COMPLETED 0
#define ST_MAX_STEPS -100
#define ST_UNATTAINABLE -300
#define ST_END_REACHED -2
#define ST_END_UNREACHABLE -3
#define ST_INVALID_FORM -400

enum { C_M = 0, C_I1 = 1, C_D1 = 2, C_I2 = 3, C_D2 = 4, NCOMP = 5 };

/* wavefront/wavefront_heuristic.h:41-49 */
enum {
  HS_BANDED_STATIC = 0x01,
  HS_BANDED_ADAPTIVE = 0x02,
  HS_WFADAPTIVE = 0x04,
  HS_XDROP = 0x10,
  HS_ZDROP = 0x20,
  HS_WFMASH = 0x40,
};

typedef struct {
  int metric; /* 3 affine, 4 affine2p */
  int match, x, o1, e1, o2, e2;
  int scope; /* max_score_scope */
  int score_only;
  int max_steps;
  /* heuristic strategy: a bit set of the reference's wf_heuristic_strategy
   * values (wavefront/wavefront_heuristic.h:41-49), 0 for none, and its
   * parameters (wavefront/wavefront_heuristic.h:51-69) */
  int heur, h_min_len, h_max_dist, h_steps;
  int h_xdrop, h_zdrop, h_min_k, h_max_k;
  /* the user's penalties, as maximal-score trimming reads them
   * (wavefront/wavefront_aligner.c:664-676) */
  int um, ux, uo1, ue1, uo2, ue2;
  /* alignment form (wavefront/wavefront_attributes.h:55-69) */
  int endsfree, extension, pbf, pef, tbf, tef;
} pen_t;

typedef struct {
  int exists;   /* wavefront stored for this score/component */
  int null;     /* wavefront->null after trimming */
  int cut_null; /* null because a heuristic cut emptied it */
  int lo, hi;   /* trimmed limits */
  int ilo, ihi; /* NULL-initialised window (wf_elements_init_min/max) */
  int32_t* off; /* off[k] addressable for every k of the allocated range */
} orow_t;

typedef struct {
  int32_t* mem;
  int64_t cap, used;
} chunk_t;

typedef struct {
  int32_t* mem; /* buffer */
  int lo, hi;   /* covered diagonals */
} kbuf_t;

typedef struct {
  orow_t* rows; /* per score, per component */
  int rows_cap; /* in scores */
  chunk_t* chunks; /* chunked bump arena (chunks never move) */
  int nchunks, cur;
  int hlo, hhi;   /* historic allocation bounds of the current pair */
  int modular;    /* score-only: rows live in a ring of max_score_scope slots */
  int scope;
  kbuf_t* slotbuf; /* modular mode: one buffer per (slot, component) */
  kbuf_t nullbuf; /* all-NULL row (the reference's wavefront_null) */
  kbuf_t victim;  /* sink for non-allocated I/D outputs (wavefront_victim) */
} oracle_ws_t;

/* Unidirectional stepper: an alignment of P against T that begins in
 * component cb and ends in component ce (C_M, C_I1, C_D1, C_I2, C_D2). */
typedef struct {
  oracle_ws_t* ws;
  const pen_t* p;
  const char* P;
  int plen;
  const char* T;
  int tlen;
  int cb, ce;
  int s, null_steps, k_end;
  /* cut-off state, as wavefront_heuristic_clear leaves it at the start of
   * each alignment (wavefront/wavefront_heuristic.c:114-121) */
  int heur, steps_wait;
  int max_sw, max_sw_k, max_wf_score;
  int32_t max_sw_off;
  int zdropped; /* z-drop ended the alignment at (end_k, end_off) */
  /* the back-trace took a source from a wavefront that a cut emptied: the
   * reference's compute step read that wavefront as NULL, its back-trace
   * reads the cells (wavefront/wavefront_backtrace.c:63-75) */
  int stale_source;
  int64_t cells, ext;
  /* ends-free form of this alignment (0: end-to-end) and the free lengths after
   * the per-pair presets; the end position found by termination
   * (wf_aligner->alignment_end_pos) */
  int endsfree, pbf, pef, tbf, tef;
  int end_k;
  int32_t end_off;
} oracle_ua_t;

void oracle_ua_start(oracle_ua_t* ua, oracle_ws_t* ws, const pen_t* p, const char* P, int plen,
                     const char* T, int tlen, int cb, int ce);
/* Ends-free variant of oracle_ua_start (component M at both ends). */
void oracle_ua_start_endsfree(oracle_ua_t* ua, oracle_ws_t* ws, const pen_t* p, const char* P,
                              int plen, const char* T, int tlen, int pbf, int pef, int tbf,
                              int tef);
int oracle_ua_extend(oracle_ua_t* ua, int* max_ak);
void oracle_ua_compute(oracle_ua_t* ua);
int oracle_ua_backtrace(oracle_ua_t* ua, char* ops);
int oracle_classic_score(const pen_t* p, int plen, int tlen, int s);
/* Wavefront row (s,c) of a stepper's workspace. */
const orow_t* oracle_row(oracle_ws_t* ws, int s, int c);
void oracle_ws_init(oracle_ws_t* ws, int modular, int scope);
void oracle_ws_free(oracle_ws_t* ws);

/* One unidirectional end-to-end alignment (high-memory semantics). */
void oracle_align_one(oracle_ws_t* ws, const pen_t* p, const char* P, int plen, const char* T,
                      int tlen, int32_t* out_score, int32_t* out_status, char* ops,
                      int32_t* ops_len, int64_t* cells, int64_t* ext, int32_t* end,
                      int32_t* flags);

/* BiWFA (ultralow memory mode). */
void oracle_bialign(const pen_t* p, const char* P, int plen, const char* T, int tlen,
                    oracle_ws_t* ws, int32_t* out_score, int32_t* out_status, char* ops,
                    int32_t* ops_len, int64_t* cells, int64_t* ext, int32_t* end);

#endif /* WFA_ORACLE_INTERNAL_H_ */

/*
 * wfa_aligner.c -- host C layer of the drop-in `wavefront_aligner` API.
 *
 * Mirrors the reference's public behaviour (smarco/WFA2-lib wavefront/wfa.h):
 * attribute defaults, penalty validation and transform, status codes and the
 * cigar_t result contract.  The alignment itself is always done by the GPU
 * engine (wfa_engine.cu); there is no CPU fallback.
 */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wfa2gpu.h"
#include "wfa_engine.h"

/* wavefront/wavefront_attributes.c:38-100 -- identical default values */
wavefront_aligner_attr_t wavefront_aligner_attr_default = {
    .distance_metric = gap_affine,
    .alignment_scope = compute_alignment,
    .alignment_form =
        {
            .span = alignment_end2end,
            .extension = false,
            .pattern_begin_free = 0,
            .pattern_end_free = 0,
            .text_begin_free = 0,
            .text_end_free = 0,
        },
    .linear_penalties = {.match = 0, .mismatch = 4, .indel = 2},
    .affine_penalties = {.match = 0, .mismatch = 4, .gap_opening = 6, .gap_extension = 2},
    .affine2p_penalties = {.match = 0,
                           .mismatch = 4,
                           .gap_opening1 = 6,
                           .gap_extension1 = 2,
                           .gap_opening2 = 24,
                           .gap_extension2 = 1},
    .heuristic =
        {
            .strategy = wf_heuristic_wfadaptive,
            .min_wavefront_length = 10,
            .max_distance_threshold = 50,
            .steps_between_cutoffs = 1,
        },
    .memory_mode = wavefront_memory_high,
    .mm_allocator = NULL,
    .plot = {.enabled = false, .resolution_points = 2000, .align_level = 0},
    .system =
        {
            .max_alignment_steps = INT_MAX,
            .probe_interval_global = 3000,
            .probe_interval_compact = 6000,
            .max_memory_compact = (uint64_t)-1,
            .max_memory_resident = (uint64_t)-1,
            .max_memory_abort = UINT64_MAX,
            .verbose = 0,
            .check_alignment_correct = false,
            .max_num_threads = 1,
            .min_offsets_per_thread = 500,
        },
};

/* wavefront/wavefront_aligner.c:40-101 -- same messages */
char* wavefront_align_strerror(const int error_code) {
  switch (error_code) {
    case WF_STATUS_ALG_COMPLETED: return "[WFA] Alignment completed successfully";
    case WF_STATUS_ALG_PARTIAL: return "[WFA] Alignment extension computed (partial alignment)";
    case WF_STATUS_MAX_STEPS_REACHED: return "[WFA] Alignment failed. Maximum WFA-steps limit reached";
    case WF_STATUS_OOM: return "[WFA] Alignment failed. Maximum memory limit reached";
    case WF_STATUS_UNATTAINABLE: return "[WFA] Alignment failed. Unattainable under configured heuristics";
    case WF_STATUS_END_REACHED: return "[WFA] Alignment end reached";
    case WF_STATUS_END_UNREACHABLE:
      return "[WFA] Alignment end unreachable under current configuration (due to heuristics like Z-drop)";
    default: return "[WFA] Unknown error code";
  }
}
char* wavefront_align_strerror_short(const int error_code) {
  switch (error_code) {
    case WF_STATUS_ALG_COMPLETED: return "OK.Full";
    case WF_STATUS_ALG_PARTIAL: return "OK.Partial";
    case WF_STATUS_MAX_STEPS_REACHED: return "FAILED.MaxWFASteps";
    case WF_STATUS_OOM: return "FAILED.OOM";
    case WF_STATUS_UNATTAINABLE: return "FAILED.Unattainable";
    case WF_STATUS_END_REACHED: return "INTERNAL.Reached";
    case WF_STATUS_END_UNREACHABLE: return "INTERNAL.Dropped";
    default: return "Unknown";
  }
}

/* ------------------------------------------------------------ penalties */
/* wavefront/wavefront_penalties.c:95-173 (same checks, messages and exit) */
static void penalties_set_affine(wavefront_penalties_t* wp, const affine_penalties_t* ap) {
  wp->distance_metric = gap_affine;
  if (ap->match > 0) {
    fprintf(stderr, "[WFA::Penalties] Match score must be negative or zero (M=%d)\n", ap->match);
    exit(1);
  } else if (ap->mismatch <= 0 || ap->gap_opening < 0 || ap->gap_extension <= 0) {
    fprintf(stderr, "[WFA::Penalties] Penalties (X=%d,O=%d,E=%d) must be (X>0,O>=0,E>0)\n",
            ap->mismatch, ap->gap_opening, ap->gap_extension);
    exit(1);
  }
  if (ap->match < 0) {
    wp->match = ap->match;
    wp->mismatch = 2 * ap->mismatch - 2 * ap->match;
    wp->gap_opening1 = 2 * ap->gap_opening;
    wp->gap_extension1 = 2 * ap->gap_extension - ap->match;
  } else {
    wp->match = 0;
    wp->mismatch = ap->mismatch;
    wp->gap_opening1 = ap->gap_opening;
    wp->gap_extension1 = ap->gap_extension;
  }
  wp->gap_opening2 = -1;
  wp->gap_extension2 = -1;
  wp->affine_penalties = *ap;
  wp->internal_gap_e = ap->gap_extension;
}
static void penalties_set_affine2p(wavefront_penalties_t* wp, const affine2p_penalties_t* ap) {
  wp->distance_metric = gap_affine_2p;
  if (ap->match > 0) {
    fprintf(stderr, "[WFA::Penalties] Match score must be negative or zero (M=%d)\n", ap->match);
    exit(1);
  } else if (ap->mismatch <= 0 || ap->gap_opening1 < 0 || ap->gap_extension1 <= 0 ||
             ap->gap_opening2 < 0 || ap->gap_extension2 <= 0) {
    fprintf(stderr,
            "[WFA::Penalties] Penalties (X=%d,O1=%d,E1=%d,O2=%d,E2=%d) must be "
            "(X>0,O1>=0,E1>0,O2>=0,E2>0)\n",
            ap->mismatch, ap->gap_opening1, ap->gap_extension1, ap->gap_opening2,
            ap->gap_extension2);
    exit(1);
  }
  if (ap->match < 0) {
    wp->match = ap->match;
    wp->mismatch = 2 * ap->mismatch - 2 * ap->match;
    wp->gap_opening1 = 2 * ap->gap_opening1;
    wp->gap_extension1 = 2 * ap->gap_extension1 - ap->match;
    wp->gap_opening2 = 2 * ap->gap_opening2;
    wp->gap_extension2 = 2 * ap->gap_extension2 - ap->match;
  } else {
    wp->match = 0;
    wp->mismatch = ap->mismatch;
    wp->gap_opening1 = ap->gap_opening1;
    wp->gap_extension1 = ap->gap_extension1;
    wp->gap_opening2 = ap->gap_opening2;
    wp->gap_extension2 = ap->gap_extension2;
  }
  wp->affine2p_penalties = *ap;
  wp->internal_gap_e = ap->gap_extension1;
}
/* edit / indel / gap-linear keep the reference's representation
 * (wavefront/wavefront_penalties.c:37-94). */
static void penalties_set_other(wavefront_penalties_t* wp, const wavefront_aligner_attr_t* a) {
  memset(wp, 0, sizeof(*wp));
  wp->distance_metric = a->distance_metric;
  if (a->distance_metric == gap_linear) {
    const linear_penalties_t* lp = &a->linear_penalties;
    if (lp->match > 0) {
      fprintf(stderr, "[WFA::Penalties] Match score must be negative or zero (M=%d)\n", lp->match);
      exit(1);
    } else if (lp->mismatch <= 0 || lp->indel <= 0) {
      fprintf(stderr, "[WFA::Penalties] Penalties (X=%d,D=%d,I=%d) must be (X>0,D>0,I>0)\n",
              lp->mismatch, lp->indel, lp->indel);
      exit(1);
    }
    wp->linear_penalties = *lp;
    wp->match = lp->match;
    wp->mismatch = lp->match < 0 ? 2 * lp->mismatch - 2 * lp->match : lp->mismatch;
    wp->gap_opening1 = lp->match < 0 ? 2 * lp->indel - lp->match : lp->indel;
    wp->internal_gap_e = lp->indel;
  } else {
    wp->mismatch = (a->distance_metric == edit) ? 1 : -1;
    wp->gap_opening1 = 1;
  }
  wp->gap_extension1 = -1;
  wp->gap_opening2 = -1;
  wp->gap_extension2 = -1;
}

/* ----------------------------------------------------------------- setup */
wavefront_aligner_t* wavefront_aligner_new(wavefront_aligner_attr_t* attributes) {
  if (attributes == NULL) attributes = &wavefront_aligner_attr_default;
  wavefront_aligner_t* wf = (wavefront_aligner_t*)calloc(1, sizeof(wavefront_aligner_t));
  if (!wf) return NULL;
  wf->align_mode =
      (attributes->memory_mode == wavefront_memory_ultralow) ? wf_align_biwfa : wf_align_regular;
  wf->align_mode_tag = NULL;
  wf->alignment_scope = attributes->alignment_scope;
  wf->alignment_form = attributes->alignment_form;
  switch (attributes->distance_metric) {
    case gap_affine: penalties_set_affine(&wf->penalties, &attributes->affine_penalties); break;
    case gap_affine_2p: penalties_set_affine2p(&wf->penalties, &attributes->affine2p_penalties); break;
    default: penalties_set_other(&wf->penalties, attributes); break;
  }
  wf->heuristic = attributes->heuristic;
  wf->memory_mode = attributes->memory_mode;
  wf->system = attributes->system;
  const int score_only = (attributes->alignment_scope == compute_score);
  wf->cigar = cigar_new(score_only ? 10 : 2 * (1000 + 1000));
  wf->align_status.status = WF_STATUS_OK;
  int err = 0;
  wf->engine = wf2g_engine_new(&err);
  return wf;
}

void wavefront_aligner_reap(wavefront_aligner_t* const wf_aligner) {
  (void)wf_aligner; /* device buffers are reused across calls; nothing to trim */
}

void wavefront_aligner_delete(wavefront_aligner_t* const wf_aligner) {
  if (!wf_aligner) return;
  wf2g_engine_free(wf_aligner->engine);
  cigar_free(wf_aligner->cigar);
  free(wf_aligner);
}

/* ------------------------------------------------------------- setters */
/* wavefront/wavefront_aligner.c:508-645 */
void wavefront_aligner_set_alignment_end_to_end(wavefront_aligner_t* const wf) {
  wf->alignment_form.span = alignment_end2end;
  wf->alignment_form.extension = false;
}
void wavefront_aligner_set_alignment_free_ends(wavefront_aligner_t* const wf,
                                               const int pattern_begin_free,
                                               const int pattern_end_free,
                                               const int text_begin_free,
                                               const int text_end_free) {
  wf->alignment_form.span = alignment_endsfree;
  wf->alignment_form.extension = false;
  wf->alignment_form.pattern_begin_free = pattern_begin_free;
  wf->alignment_form.pattern_end_free = pattern_end_free;
  wf->alignment_form.text_begin_free = text_begin_free;
  wf->alignment_form.text_end_free = text_end_free;
}
void wavefront_aligner_set_alignment_extension(wavefront_aligner_t* const wf) {
  wf->alignment_form.span = alignment_endsfree;
  wf->alignment_form.extension = true;
}
/* The setters add a strategy to the set, as the reference's do
 * (wavefront/wavefront_heuristic.c:40-113); only "none" clears it.  One
 * steps_between_cutoffs serves every strategy of the set. */
void wavefront_aligner_set_heuristic_none(wavefront_aligner_t* const wf) {
  wf->heuristic.strategy = wf_heuristic_none;
}
void wavefront_aligner_set_heuristic_wfadaptive(wavefront_aligner_t* const wf,
                                                const int min_wavefront_length,
                                                const int max_distance_threshold,
                                                const int score_steps) {
  wf->heuristic.strategy |= wf_heuristic_wfadaptive;
  wf->heuristic.min_wavefront_length = min_wavefront_length;
  wf->heuristic.max_distance_threshold = max_distance_threshold;
  wf->heuristic.steps_between_cutoffs = score_steps;
}
void wavefront_aligner_set_heuristic_wfmash(wavefront_aligner_t* const wf,
                                            const int min_wavefront_length,
                                            const int max_distance_threshold,
                                            const int score_steps) {
  wf->heuristic.strategy |= wf_heuristic_wfmash;
  wf->heuristic.min_wavefront_length = min_wavefront_length;
  wf->heuristic.max_distance_threshold = max_distance_threshold;
  wf->heuristic.steps_between_cutoffs = score_steps;
}
void wavefront_aligner_set_heuristic_xdrop(wavefront_aligner_t* const wf, const int xdrop,
                                           const int score_steps) {
  wf->heuristic.strategy |= wf_heuristic_xdrop;
  wf->heuristic.xdrop = xdrop;
  wf->heuristic.steps_between_cutoffs = score_steps;
}
void wavefront_aligner_set_heuristic_zdrop(wavefront_aligner_t* const wf, const int ydrop,
                                           const int score_steps) {
  wf->heuristic.strategy |= wf_heuristic_zdrop;
  wf->heuristic.zdrop = ydrop;
  wf->heuristic.steps_between_cutoffs = score_steps;
}
void wavefront_aligner_set_heuristic_banded_static(wavefront_aligner_t* const wf,
                                                   const int band_min_k, const int band_max_k) {
  wf->heuristic.strategy |= wf_heuristic_banded_static;
  wf->heuristic.min_k = band_min_k;
  wf->heuristic.max_k = band_max_k;
}
void wavefront_aligner_set_heuristic_banded_adaptive(wavefront_aligner_t* const wf,
                                                     const int band_min_k, const int band_max_k,
                                                     const int score_steps) {
  wf->heuristic.strategy |= wf_heuristic_banded_adaptive;
  wf->heuristic.min_k = band_min_k;
  wf->heuristic.max_k = band_max_k;
  wf->heuristic.steps_between_cutoffs = score_steps;
}
void wavefront_aligner_set_max_alignment_steps(wavefront_aligner_t* const wf,
                                               const int max_alignment_steps) {
  wf->system.max_alignment_steps = max_alignment_steps;
}
void wavefront_aligner_set_max_memory(wavefront_aligner_t* const wf,
                                      const uint64_t max_memory_resident,
                                      const uint64_t max_memory_abort) {
  wf->system.max_memory_resident = max_memory_resident;
  wf->system.max_memory_abort = max_memory_abort;
}
void wavefront_aligner_set_max_num_threads(wavefront_aligner_t* const wf,
                                           const int max_num_threads) {
  wf->system.max_num_threads = max_num_threads;
}
void wavefront_aligner_set_min_offsets_per_thread(wavefront_aligner_t* const wf,
                                                  const int min_offsets_per_thread) {
  wf->system.min_offsets_per_thread = min_offsets_per_thread;
}

/* ----------------------------------------------------------------- align */
/* Returns 0 and fills cfg when the aligner's configuration is computed on the
 * GPU; otherwise the WF_STATUS_* / WF2G_ERR_* code to report. */
static int make_cfg(const wavefront_aligner_t* wf, wf2g_cfg_t* cfg) {
  const wavefront_penalties_t* p = &wf->penalties;
  const int lin = p->distance_metric <= gap_linear;  /* indel, edit, gap-linear */
  const alignment_form_t* form = &wf->alignment_form;
  /* extension is an ends-free form (wavefront/wavefront_aligner.c:526-530) */
  if (form->span == alignment_end2end && form->extension) return -1;
  /* the heuristic cut-offs (wavefront/wavefront_heuristic.c:506-563): one of
   * wf-adaptive/wfmash, one of x-drop/z-drop, one of banded static/adaptive */
  const int strategy = (int)wf->heuristic.strategy;
  /* drops with edit/indel: the reference exits (wavefront/wavefront_align.c:83-89) */
  if ((strategy & (wf_heuristic_xdrop | wf_heuristic_zdrop)) && p->distance_metric <= edit)
    return -1;
  /* BiWFA's searches inherit the heuristic (wavefront/wavefront_bialigner.c:
   * 48-56); z-drop is not computed there */
  if (wf->memory_mode == wavefront_memory_ultralow && (strategy & wf_heuristic_zdrop))
    return -1;
  cfg->metric = (int)p->distance_metric;
  cfg->match = p->match;
  cfg->x = p->mismatch;
  cfg->o1 = p->gap_opening1;
  cfg->e1 = lin ? 0 : p->gap_extension1;
  cfg->o2 = lin ? 0 : p->gap_opening2;
  cfg->e2 = lin ? 0 : p->gap_extension2;
  cfg->score_only = (wf->alignment_scope == compute_score);
  cfg->max_steps = wf->system.max_alignment_steps > 0 ? wf->system.max_alignment_steps : INT_MAX;
  /* ultralow memory mode is BiWFA (wavefront/wavefront_align.c:138-146) */
  cfg->ultralow = (wf->memory_mode == wavefront_memory_ultralow);
  cfg->heur = strategy;
  cfg->h_min_len = wf->heuristic.min_wavefront_length;
  cfg->h_max_dist = wf->heuristic.max_distance_threshold;
  cfg->h_steps = wf->heuristic.steps_between_cutoffs;
  cfg->h_xdrop = wf->heuristic.xdrop;
  cfg->h_zdrop = wf->heuristic.zdrop;
  cfg->h_min_k = wf->heuristic.min_k;
  cfg->h_max_k = wf->heuristic.max_k;
  /* alignment form (wavefront/wavefront_attributes.h:55-69) */
  cfg->endsfree = (form->span == alignment_endsfree);
  cfg->extension = cfg->endsfree && form->extension;
  cfg->pbf = cfg->endsfree ? form->pattern_begin_free : 0;
  cfg->pef = cfg->endsfree ? form->pattern_end_free : 0;
  cfg->tbf = cfg->endsfree ? form->text_begin_free : 0;
  cfg->tef = cfg->endsfree ? form->text_end_free : 0;
  if (cfg->endsfree) {
    /* BiWFA has no ends-free form (the reference exits,
     * wavefront/wavefront_align.c:67-82) */
    if (cfg->ultralow) return -1;
    if (cfg->pbf < 0 || cfg->pef < 0 || cfg->tbf < 0 || cfg->tef < 0) return -1;
    /* edit and indel never widen the score-0 wavefront's initialised window
     * (wavefront/wavefront_compute_edit.c:321-374), so their back-trace reads
     * begin-free diagonals as sourceless and can end in matches over
     * mismatches: a full alignment is not computed.  The score-only search
     * is (it reads those cells by their limits). */
    if (!cfg->extension && !cfg->score_only && p->distance_metric <= edit &&
        (cfg->pbf > 0 || cfg->tbf > 0))
      return -1;
  }
  /* the user's penalties, for maximal-score trimming (wavefront/wavefront_aligner.c:664-676) */
  if (lin) {
    cfg->um = p->linear_penalties.match;
    cfg->ux = p->linear_penalties.mismatch;
    cfg->uo1 = p->linear_penalties.indel;
    cfg->ue1 = cfg->uo2 = cfg->ue2 = 0;
  } else if (p->distance_metric == gap_affine) {
    cfg->um = p->affine_penalties.match;
    cfg->ux = p->affine_penalties.mismatch;
    cfg->uo1 = p->affine_penalties.gap_opening;
    cfg->ue1 = p->affine_penalties.gap_extension;
    cfg->uo2 = cfg->ue2 = 0;
  } else {
    cfg->um = p->affine2p_penalties.match;
    cfg->ux = p->affine2p_penalties.mismatch;
    cfg->uo1 = p->affine2p_penalties.gap_opening1;
    cfg->ue1 = p->affine2p_penalties.gap_extension1;
    cfg->uo2 = p->affine2p_penalties.gap_opening2;
    cfg->ue2 = p->affine2p_penalties.gap_extension2;
  }
  return 0;
}

/* WFA score from the classic score (inverse of wavefront/wavefront_compute.c:108-120) */
static int wf_score_of(const wavefront_aligner_t* wf, int classic, int plen, int tlen) {
  if (wf->penalties.match == 0) return -classic;
  return (-wf->penalties.match) * (plen + tlen) - 2 * classic;
}

static int warned_config = 0;

static int align_one(wavefront_aligner_t* const wf, const char* seqbuf, int plen, int tlen) {
  cigar_t* const cigar = wf->cigar;
  cigar_clear(cigar);
  wf2g_cfg_t cfg;
  if (make_cfg(wf, &cfg) != 0) {
    if (!warned_config) {
      fprintf(stderr,
              "[wfa2gpu] configuration not computed on the GPU (drops with edit/indel; "
              "BiWFA with a heuristic other than wf-adaptive or with free ends; begin-free "
              "lengths with match < 0 or edit/indel)\n");
      warned_config = 1;
    }
    wf->align_status.status = WF_STATUS_UNATTAINABLE;
    return WF_STATUS_UNATTAINABLE;
  }
  if (!wf->engine) {
    fprintf(stderr, "[wfa2gpu] no usable GPU: alignment not computed\n");
    wf->align_status.status = WF_STATUS_UNATTAINABLE;
    return WF_STATUS_UNATTAINABLE;
  }
  /* wavefront/wavefront_align.c:90-101: the same check, message and exit */
  if (cfg.endsfree && !cfg.extension &&
      (cfg.pbf > plen || cfg.pef > plen || cfg.tbf > tlen || cfg.tef > tlen)) {
    fprintf(stderr,
            "[WFA] Ends-free parameters must be not larger than the sequences "
            "(P0=%d,Pf=%d,T0=%d,Tf=%d). Must be (P0<=|P|,Pf<=|P|,T0<=|T|,Tf<=|T|) where "
            "(|P|,|T|)=(%d,%d)\n",
            cfg.pbf, cfg.pef, cfg.tbf, cfg.tef, plen, tlen);
    exit(1);
  }
  const int score_only = cfg.score_only;
  if (!score_only) cigar_resize(cigar, 2 * (plen + tlen) + 1);
  const int64_t p_off = 0, t_off = plen, ops_off = 0;
  int32_t score = 0, status = 0, ops_len = 0, end_info[3] = {-1, -1, 0};
  const int rc = wf2g_engine_align(wf->engine, &cfg, 1, 0, seqbuf, &p_off, &plen, &t_off, &tlen,
                                   0, &score, &status, score_only ? NULL : cigar->operations,
                                   score_only ? NULL : &ops_off, score_only ? NULL : &ops_len,
                                   end_info, NULL);
  if (rc != 0) {
    wf->align_status.status = WF_STATUS_UNATTAINABLE;
    return WF_STATUS_UNATTAINABLE;
  }
  wf->align_status.status = status;
  if (status == WF_STATUS_ALG_COMPLETED || status == WF_STATUS_ALG_PARTIAL) {
    cigar->score = score;
    if (cfg.ultralow) {
      /* the lengths where the reference sets them (a score-only search, or a
       * full alignment whose top level split at a breakpoint), else -1 */
      cigar->end_v = end_info[0];
      cigar->end_h = end_info[1];
      wf->align_status.score = wf_score_of(wf, score, plen, tlen);
    } else {
      cigar->end_v = end_info[0];
      cigar->end_h = end_info[1];
      wf->align_status.score = end_info[2];
    }
    if (!score_only) {
      cigar->begin_offset = 0;
      cigar->end_offset = ops_len;
      cigar->operations[ops_len] = '\0';
    }
  } else if (status == WF_STATUS_MAX_STEPS_REACHED) {
    cigar->score = -wf->system.max_alignment_steps;
    wf->align_status.score = wf->system.max_alignment_steps;
  }
  return status;
}

int wavefront_align(wavefront_aligner_t* const wf_aligner, const char* const pattern,
                    const int pattern_length, const char* const text, const int text_length) {
  if (pattern_length < 0 || text_length < 0) {
    wf_aligner->align_status.status = WF_STATUS_UNATTAINABLE;
    return WF_STATUS_UNATTAINABLE;
  }
  char* buf = (char*)malloc((size_t)pattern_length + text_length + 16);
  memcpy(buf, pattern, (size_t)pattern_length);
  memcpy(buf + pattern_length, text, (size_t)text_length);
  const int st = align_one(wf_aligner, buf, pattern_length, text_length);
  free(buf);
  return st;
}

int wavefront_align_lambda(wavefront_aligner_t* const wf_aligner,
                           alignment_match_funct_t const match_funct, void* match_funct_arguments,
                           const int pattern_length, const int text_length) {
  (void)match_funct;
  (void)match_funct_arguments;
  (void)pattern_length;
  (void)text_length;
  fprintf(stderr, "[wfa2gpu] wavefront_align_lambda: a host match function cannot run on the GPU\n");
  cigar_clear(wf_aligner->cigar);
  wf_aligner->align_status.status = WF_STATUS_UNATTAINABLE;
  return WF_STATUS_UNATTAINABLE;
}

int wavefront_align_packed2bits(wavefront_aligner_t* const wf_aligner,
                                const uint8_t* const pattern, const int pattern_length,
                                const uint8_t* const text, const int text_length) {
  static const char dec[4] = {'A', 'C', 'G', 'T'};
  if (pattern_length < 0 || text_length < 0) {
    wf_aligner->align_status.status = WF_STATUS_UNATTAINABLE;
    return WF_STATUS_UNATTAINABLE;
  }
  char* buf = (char*)malloc((size_t)pattern_length + text_length + 16);
  for (int i = 0; i < pattern_length; ++i) buf[i] = dec[(pattern[i >> 2] >> (2 * (i & 3))) & 3];
  for (int i = 0; i < text_length; ++i)
    buf[pattern_length + i] = dec[(text[i >> 2] >> (2 * (i & 3))) & 3];
  const int st = align_one(wf_aligner, buf, pattern_length, text_length);
  free(buf);
  return st;
}

/* ----------------------------------------------------------------- batch */
int wavefront_align_batch(wavefront_aligner_t* const wf_aligner, const int num_pairs,
                          const char* seqs, const int64_t* pattern_offsets,
                          const int32_t* pattern_lengths, const int64_t* text_offsets,
                          const int32_t* text_lengths, int32_t* scores, int32_t* status,
                          char* cigar_ops, const int64_t* cigar_offsets, int32_t* cigar_lengths) {
  if (!wf_aligner || num_pairs < 0) return WF2G_ERR_ARGS;
  if (!wf_aligner->engine) return WF2G_ERR_NO_GPU;
  wf2g_cfg_t cfg;
  if (make_cfg(wf_aligner, &cfg) != 0) return WF2G_ERR_CONFIG;
  if (!cfg.score_only && (!cigar_ops || !cigar_offsets || !cigar_lengths)) return WF2G_ERR_ARGS;
  return wf2g_engine_align(wf_aligner->engine, &cfg, num_pairs, 0, seqs, pattern_offsets,
                           pattern_lengths, text_offsets, text_lengths, 0, scores, status,
                           cfg.score_only ? NULL : cigar_ops, cfg.score_only ? NULL : cigar_offsets,
                           cfg.score_only ? NULL : cigar_lengths, NULL, NULL);
}

int wavefront_align_batch_ends(wavefront_aligner_t* const wf_aligner, const int num_pairs,
                               const char* seqs, const int64_t* pattern_offsets,
                               const int32_t* pattern_lengths, const int64_t* text_offsets,
                               const int32_t* text_lengths, int32_t* scores, int32_t* status,
                               char* cigar_ops, const int64_t* cigar_offsets,
                               int32_t* cigar_lengths, int32_t* end_info) {
  if (!wf_aligner || num_pairs < 0 || !end_info) return WF2G_ERR_ARGS;
  if (!wf_aligner->engine) return WF2G_ERR_NO_GPU;
  wf2g_cfg_t cfg;
  if (make_cfg(wf_aligner, &cfg) != 0) return WF2G_ERR_CONFIG;
  if (cfg.ultralow) return WF2G_ERR_CONFIG;
  if (!cfg.score_only && (!cigar_ops || !cigar_offsets || !cigar_lengths)) return WF2G_ERR_ARGS;
  return wf2g_engine_align(wf_aligner->engine, &cfg, num_pairs, 0, seqs, pattern_offsets,
                           pattern_lengths, text_offsets, text_lengths, 0, scores, status,
                           cfg.score_only ? NULL : cigar_ops, cfg.score_only ? NULL : cigar_offsets,
                           cfg.score_only ? NULL : cigar_lengths, end_info, NULL);
}

int wavefront_align_batch_device(wavefront_aligner_t* const wf_aligner, const int num_pairs,
                                 const char* d_seqs, const int64_t* d_pattern_offsets,
                                 const int32_t* d_pattern_lengths, const int64_t* d_text_offsets,
                                 const int32_t* d_text_lengths, const int max_sequence_length,
                                 int32_t* d_scores, int32_t* d_status, char* d_cigar_ops,
                                 const int64_t* d_cigar_offsets, int32_t* d_cigar_lengths,
                                 void* cuda_stream) {
  if (!wf_aligner || num_pairs < 0) return WF2G_ERR_ARGS;
  if (!wf_aligner->engine) return WF2G_ERR_NO_GPU;
  wf2g_cfg_t cfg;
  if (make_cfg(wf_aligner, &cfg) != 0) return WF2G_ERR_CONFIG;
  if (!cfg.score_only && (!d_cigar_ops || !d_cigar_offsets || !d_cigar_lengths)) return WF2G_ERR_ARGS;
  return wf2g_engine_align(wf_aligner->engine, &cfg, num_pairs, 1, d_seqs, d_pattern_offsets,
                           d_pattern_lengths, d_text_offsets, d_text_lengths, max_sequence_length,
                           d_scores, d_status, cfg.score_only ? NULL : d_cigar_ops,
                           cfg.score_only ? NULL : d_cigar_offsets,
                           cfg.score_only ? NULL : d_cigar_lengths, NULL, cuda_stream);
}

int wavefront_align_batch_device_noalloc(wavefront_aligner_t* const wf_aligner,
                                         const int num_pairs, const char* d_seqs,
                                         const int64_t* d_pattern_offsets,
                                         const int32_t* d_pattern_lengths,
                                         const int64_t* d_text_offsets,
                                         const int32_t* d_text_lengths,
                                         const int max_sequence_length, int32_t* d_scores,
                                         int32_t* d_status, char* d_cigar_ops,
                                         const int64_t* d_cigar_offsets, int32_t* d_cigar_lengths,
                                         void* cuda_stream) {
  if (!wf_aligner || num_pairs < 0) return WF2G_ERR_ARGS;
  const int dev = wf2g_engine_device();
  if (dev < 0) return WF2G_ERR_NO_GPU;
  /* the call runs on the current device: it must be the aligner's */
  if (wf_aligner->engine && wf2g_engine_owner_device(wf_aligner->engine) != dev)
    return WF2G_ERR_ARGS;
  wf2g_cfg_t cfg;
  if (make_cfg(wf_aligner, &cfg) != 0) return WF2G_ERR_CONFIG;
  return wf2g_noalloc_align(&cfg, num_pairs, d_seqs, d_pattern_offsets, d_pattern_lengths,
                            d_text_offsets, d_text_lengths, max_sequence_length, d_scores,
                            d_status, cfg.score_only ? NULL : d_cigar_ops,
                            cfg.score_only ? NULL : d_cigar_offsets,
                            cfg.score_only ? NULL : d_cigar_lengths, cuda_stream);
}

int64_t wavefront_aligner_gpu_launches(const wavefront_aligner_t* const wf_aligner) {
  return wf_aligner ? wf2g_engine_launches(wf_aligner->engine) : 0;
}

int wfa2gpu_device(void) { return wf2g_engine_device(); }

/* ----------------------------------------------------------------- serving */
wavefront_server_t* wavefront_server_new(const wavefront_aligner_t* const wf_aligner,
                                         const wavefront_server_attr_t* const attributes) {
  if (!wf_aligner) return NULL;
  wf2g_cfg_t cfg;
  if (make_cfg(wf_aligner, &cfg) != 0 || cfg.ultralow) {
    fprintf(stderr, "[wfa2gpu] server: configuration not served (needs gap-affine or "
                    "gap-affine-2p, end-to-end, heuristic none, memory mode high)\n");
    return NULL;
  }
  wavefront_server_attr_t a = {0, 0, 0, 0, -1, 0};
  if (attributes) a = *attributes;
  int err = 0;
  void* s = wf2g_server_new(&cfg, a.hbm_budget_bytes, a.backtrace_budget_bytes, a.lanes,
                            a.max_batch_pairs, a.batch_window_us < 0 ? 200 : a.batch_window_us,
                            a.biwfa_min_length == 0 ? 8192 : a.biwfa_min_length, &err);
  return (wavefront_server_t*)s;
}

int64_t wavefront_server_submit(wavefront_server_t* const server, const char* const pattern,
                                const int pattern_length, const char* const text,
                                const int text_length) {
  if (!server) return WF2G_ERR_ARGS;
  return wf2g_server_submit(server, pattern, pattern_length, text, text_length);
}

int wavefront_server_poll(wavefront_server_t* const server, wavefront_server_result_t* results,
                          const int max_results, const int timeout_us) {
  if (!server) return WF2G_ERR_ARGS;
  return wf2g_server_poll(server, results, max_results, timeout_us);
}

int64_t wavefront_server_in_flight(wavefront_server_t* const server) {
  return server ? wf2g_server_in_flight(server) : 0;
}

int64_t wavefront_server_gpu_launches(wavefront_server_t* const server) {
  return server ? wf2g_server_launches(server) : 0;
}

void wavefront_server_delete(wavefront_server_t* const server) {
  if (server) wf2g_server_free(server);
}

/* ------------------------------------------------------------ utilities and display */
/* wavefront/wavefront_aligner.c:647-662: the memory the aligner holds; here
 * the GPU engine's device and pinned host buffers */
uint64_t wavefront_aligner_get_size(wavefront_aligner_t* const wf_aligner) {
  return wf_aligner ? (uint64_t)wf2g_engine_bytes(wf_aligner->engine) : 0;
}
/* wavefront/wavefront_aligner.c:664-676: trims the aligner's CIGAR to its
 * maximal-score prefix under the user's penalties; edit and indel are not
 * trimmed */
bool wavefront_aligner_maxtrim_cigar(wavefront_aligner_t* const wf_aligner) {
  switch (wf_aligner->penalties.distance_metric) {
    case gap_linear:
      return cigar_maxtrim_gap_linear(wf_aligner->cigar, &wf_aligner->penalties.linear_penalties);
    case gap_affine:
      return cigar_maxtrim_gap_affine(wf_aligner->cigar, &wf_aligner->penalties.affine_penalties);
    case gap_affine_2p:
      return cigar_maxtrim_gap_affine2p(wf_aligner->cigar,
                                        &wf_aligner->penalties.affine2p_penalties);
    default:
      return false;
  }
}
/* wavefront/wavefront_aligner.c:680-735: the same labels as the reference
 * prints them */
void wavefront_aligner_print_mode(FILE* const stream, wavefront_aligner_t* const wf_aligner) {
  if (wf_aligner->align_mode_tag != NULL) fprintf(stream, "%s::", wf_aligner->align_mode_tag);
  static const char* const names[] = {"WFA", "BiWFA", "BiWFA::Forward", "BiWFA::Reverse",
                                      "BiWFA::SubWFA"};
  const int m = (int)wf_aligner->align_mode;
  fputs(m >= 1 && m <= 4 ? names[m] : names[0], stream);
}
void wavefront_aligner_print_scope(FILE* const stream, wavefront_aligner_t* const wf_aligner) {
  const char* const scope = wf_aligner->alignment_scope == compute_score ? "score" : "alignment";
  const alignment_form_t* const f = &wf_aligner->alignment_form;
  if (f->span == alignment_end2end) {
    fprintf(stream, "(%s,end2end)", scope);
  } else {
    fprintf(stream, "(%s,endsfree,%d,%d,%d,%d)", scope, f->pattern_begin_free,
            f->pattern_end_free, f->text_begin_free, f->text_end_free);
  }
}
void wavefront_aligner_print_conf(FILE* const stream, wavefront_aligner_t* const wf_aligner) {
  static const char* const modes[] = {"MHigh", "MMed", "MLow", "BiWFA"};
  const int m = (int)wf_aligner->memory_mode;
  fprintf(stream, "(%s", m >= 0 && m <= 3 ? modes[m] : "");
  if (wf_aligner->system.max_alignment_steps == INT_MAX) {
    fprintf(stream, ",inf)");
  } else {
    fprintf(stream, ",%d)", wf_aligner->system.max_alignment_steps);
  }
}

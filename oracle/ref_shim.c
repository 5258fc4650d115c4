/*
 * ref_shim.c -- flat batch driver around the UNMODIFIED reference library
 * (smarco/WFA2-lib), compiled from the reference's own sources by
 * oracle/Makefile into oracle/_ref/libwfa_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY: used to pin the CPU restatement (wfa_oracle.c)
 * and to generate golden fixtures; never part of the product library.
 *
 * It configures one aligner per host thread exactly like the reference's
 * benchmark tool does (tools/align_benchmark/align_benchmark.c:155-242 and
 * :504-586): heuristic none, the requested metric, penalties, scope and
 * memory mode, then calls wavefront_align() per pair.
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "wavefront/wavefront_align.h"

int ref_align_batch(const int* cfg, int num_pairs, const char* sequences, const int64_t* p_off,
                    const int32_t* p_len, const int64_t* t_off, const int32_t* t_len,
                    int32_t* out_score, int32_t* out_status, char* out_ops,
                    const int64_t* ops_off, int32_t* out_ops_len, int64_t* out_cells,
                    int64_t* out_ext, int32_t* out_end, int nthreads) {
  (void)out_cells;
  (void)out_ext;
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = (distance_metric_t)cfg[0];
  if (cfg[0] == gap_affine) {
    attr.affine_penalties.match = cfg[1];
    attr.affine_penalties.mismatch = cfg[2];
    attr.affine_penalties.gap_opening = cfg[3];
    attr.affine_penalties.gap_extension = cfg[4];
  } else if (cfg[0] == gap_affine_2p) {
    attr.affine2p_penalties.match = cfg[1];
    attr.affine2p_penalties.mismatch = cfg[2];
    attr.affine2p_penalties.gap_opening1 = cfg[3];
    attr.affine2p_penalties.gap_extension1 = cfg[4];
    attr.affine2p_penalties.gap_opening2 = cfg[5];
    attr.affine2p_penalties.gap_extension2 = cfg[6];
  } else if (cfg[0] == gap_linear) {
    attr.linear_penalties.match = cfg[1];
    attr.linear_penalties.mismatch = cfg[2];
    attr.linear_penalties.indel = cfg[3];
  } else if (cfg[0] != edit && cfg[0] != indel) {
    return -1;
  }
  attr.memory_mode = (wavefront_memory_t)cfg[7];
  attr.alignment_scope = cfg[8] ? compute_score : compute_alignment;
  attr.heuristic.strategy = wf_heuristic_none;
  if (cfg[10] == 1 || cfg[20] != 0) {
    /* cfg[20]: a wf_heuristic_strategy bit set; cfg[10] == 1 alone: wf-adaptive */
    attr.heuristic.strategy = cfg[20] != 0 ? (wf_heuristic_strategy)cfg[20] : wf_heuristic_wfadaptive;
    attr.heuristic.min_wavefront_length = cfg[11];
    attr.heuristic.max_distance_threshold = cfg[12];
    attr.heuristic.steps_between_cutoffs = cfg[13];
    attr.heuristic.xdrop = cfg[21];
    attr.heuristic.zdrop = cfg[22];
    attr.heuristic.min_k = cfg[23];
    attr.heuristic.max_k = cfg[24];
  }
  if (cfg[9] > 0) attr.system.max_alignment_steps = cfg[9];
  if (cfg[14] == 1) {
    attr.alignment_form.span = alignment_endsfree;
    attr.alignment_form.pattern_begin_free = cfg[15];
    attr.alignment_form.pattern_end_free = cfg[16];
    attr.alignment_form.text_begin_free = cfg[17];
    attr.alignment_form.text_end_free = cfg[18];
    attr.alignment_form.extension = cfg[19] != 0;
    /* the reference exits on ends-free values longer than a sequence
     * (wavefront/wavefront_align.c:90-101): such pairs are not handed to it */
  }
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    wavefront_aligner_attr_t a = attr;
    wavefront_aligner_t* const wf = wavefront_aligner_new(&a);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (int i = 0; i < num_pairs; ++i) {
      if (cfg[14] == 1 && !cfg[19] &&
          (cfg[15] > p_len[i] || cfg[16] > p_len[i] || cfg[17] > t_len[i] || cfg[18] > t_len[i])) {
        out_status[i] = -400; /* ORACLE_STATUS_INVALID_FORM */
        out_score[i] = 0;
        out_ops_len[i] = 0;
        if (out_end) out_end[2 * i] = out_end[2 * i + 1] = -1;
        continue;
      }
      wavefront_align(wf, sequences + p_off[i], p_len[i], sequences + t_off[i], t_len[i]);
      out_status[i] = wf->align_status.status;
      cigar_t* const cg = wf->cigar;
      out_score[i] = cg->score;
      if (out_end) {
        out_end[2 * i] = cg->end_v;
        out_end[2 * i + 1] = cg->end_h;
      }
      if (!cfg[8] && out_ops != NULL &&
          (wf->align_status.status == 0 || wf->align_status.status == 1)) {
        const int n = cg->end_offset - cg->begin_offset;
        if (n > p_len[i] + t_len[i]) {
          out_ops_len[i] = -1; /* longer than the caller's buffer */
        } else {
          memcpy(out_ops + ops_off[i], cg->operations + cg->begin_offset, (size_t)n);
          out_ops_len[i] = n;
        }
      } else {
        out_ops_len[i] = 0;
      }
    }
    wavefront_aligner_delete(wf);
  }
  return 0;
}

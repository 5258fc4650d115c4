// wfa_cpp.cpp -- the C++ WFAligner classes (include/bindings/cpp/WFAligner.hpp)
// over the C ABI of wfa2gpu.h.  Each method is the C call the reference's
// binding makes for it (bindings/cpp/WFAligner.cpp): the form is set on the
// aligner, then the pair is aligned on the GPU.  Built into
// lib/libwfa2gpu_cpp.so.
#include "bindings/cpp/WFAligner.hpp"

#include <cstring>

namespace wfa {

namespace {
wavefront_memory_t memory_of(WFAligner::MemoryModel m) {
  switch (m) {
    case WFAligner::MemoryMed: return wavefront_memory_med;
    case WFAligner::MemoryLow: return wavefront_memory_low;
    case WFAligner::MemoryUltralow: return wavefront_memory_ultralow;
    default: return wavefront_memory_high;
  }
}
}  // namespace

// ---------------------------------------------------------------- set-up
WFAligner::WFAligner(const AlignmentScope alignmentScope, const MemoryModel memoryModel)
    : attributes(wavefront_aligner_attr_default), wfAligner(nullptr) {
  attributes.memory_mode = memory_of(memoryModel);
  attributes.alignment_scope = alignmentScope == Score ? compute_score : compute_alignment;
}
WFAligner::~WFAligner() { wavefront_aligner_delete(wfAligner); }

WFAlignerIndel::WFAlignerIndel(const AlignmentScope scope, const MemoryModel memory)
    : WFAligner(scope, memory) {
  attributes.distance_metric = indel;
  wfAligner = wavefront_aligner_new(&attributes);
}
WFAlignerEdit::WFAlignerEdit(const AlignmentScope scope, const MemoryModel memory)
    : WFAligner(scope, memory) {
  attributes.distance_metric = edit;
  wfAligner = wavefront_aligner_new(&attributes);
}
WFAlignerGapLinear::WFAlignerGapLinear(const int mismatch, const int indel_penalty,
                                       const AlignmentScope scope, const MemoryModel memory)
    : WFAlignerGapLinear(0, mismatch, indel_penalty, scope, memory) {}
WFAlignerGapLinear::WFAlignerGapLinear(const int match, const int mismatch,
                                       const int indel_penalty, const AlignmentScope scope,
                                       const MemoryModel memory)
    : WFAligner(scope, memory) {
  attributes.distance_metric = gap_linear;
  attributes.linear_penalties.match = match;
  attributes.linear_penalties.mismatch = mismatch;
  attributes.linear_penalties.indel = indel_penalty;
  wfAligner = wavefront_aligner_new(&attributes);
}
WFAlignerGapAffine::WFAlignerGapAffine(const int mismatch, const int gapOpening,
                                       const int gapExtension, const AlignmentScope scope,
                                       const MemoryModel memory)
    : WFAlignerGapAffine(0, mismatch, gapOpening, gapExtension, scope, memory) {}
WFAlignerGapAffine::WFAlignerGapAffine(const int match, const int mismatch, const int gapOpening,
                                       const int gapExtension, const AlignmentScope scope,
                                       const MemoryModel memory)
    : WFAligner(scope, memory) {
  attributes.distance_metric = gap_affine;
  attributes.affine_penalties.match = match;
  attributes.affine_penalties.mismatch = mismatch;
  attributes.affine_penalties.gap_opening = gapOpening;
  attributes.affine_penalties.gap_extension = gapExtension;
  wfAligner = wavefront_aligner_new(&attributes);
}
WFAlignerGapAffine2Pieces::WFAlignerGapAffine2Pieces(
    const int mismatch, const int gapOpening1, const int gapExtension1, const int gapOpening2,
    const int gapExtension2, const AlignmentScope scope, const MemoryModel memory)
    : WFAlignerGapAffine2Pieces(0, mismatch, gapOpening1, gapExtension1, gapOpening2,
                                gapExtension2, scope, memory) {}
WFAlignerGapAffine2Pieces::WFAlignerGapAffine2Pieces(
    const int match, const int mismatch, const int gapOpening1, const int gapExtension1,
    const int gapOpening2, const int gapExtension2, const AlignmentScope scope,
    const MemoryModel memory)
    : WFAligner(scope, memory) {
  attributes.distance_metric = gap_affine_2p;
  attributes.affine2p_penalties.match = match;
  attributes.affine2p_penalties.mismatch = mismatch;
  attributes.affine2p_penalties.gap_opening1 = gapOpening1;
  attributes.affine2p_penalties.gap_extension1 = gapExtension1;
  attributes.affine2p_penalties.gap_opening2 = gapOpening2;
  attributes.affine2p_penalties.gap_extension2 = gapExtension2;
  wfAligner = wavefront_aligner_new(&attributes);
}

// ---------------------------------------------------------------- end-to-end
WFAligner::AlignmentStatus WFAligner::alignEnd2End(const char* const pattern,
                                                   const int patternLength,
                                                   const char* const text,
                                                   const int textLength) {
  wavefront_aligner_set_alignment_end_to_end(wfAligner);
  return (AlignmentStatus)wavefront_align(wfAligner, pattern, patternLength, text, textLength);
}
WFAligner::AlignmentStatus WFAligner::alignEnd2End(const std::string& pattern,
                                                   const std::string& text) {
  return alignEnd2End(pattern.c_str(), (int)pattern.length(), text.c_str(), (int)text.length());
}
WFAligner::AlignmentStatus WFAligner::alignEnd2End(const uint8_t* const pattern,
                                                   const int patternLength,
                                                   const uint8_t* const text,
                                                   const int textLength) {
  wavefront_aligner_set_alignment_end_to_end(wfAligner);
  return (AlignmentStatus)wavefront_align_packed2bits(wfAligner, pattern, patternLength, text,
                                                      textLength);
}
WFAligner::AlignmentStatus WFAligner::alignEnd2End(int (*matchFunct)(int, int, void*),
                                                   void* matchFunctArguments,
                                                   const int patternLength,
                                                   const int textLength) {
  wavefront_aligner_set_alignment_end_to_end(wfAligner);
  return (AlignmentStatus)wavefront_align_lambda(wfAligner, matchFunct, matchFunctArguments,
                                                 patternLength, textLength);
}

// ---------------------------------------------------------------- ends-free
WFAligner::AlignmentStatus WFAligner::alignEndsFree(
    const char* const pattern, const int patternLength, const int patternBeginFree,
    const int patternEndFree, const char* const text, const int textLength,
    const int textBeginFree, const int textEndFree) {
  wavefront_aligner_set_alignment_free_ends(wfAligner, patternBeginFree, patternEndFree,
                                            textBeginFree, textEndFree);
  return (AlignmentStatus)wavefront_align(wfAligner, pattern, patternLength, text, textLength);
}
WFAligner::AlignmentStatus WFAligner::alignEndsFree(const std::string& pattern,
                                                    const int patternBeginFree,
                                                    const int patternEndFree,
                                                    const std::string& text,
                                                    const int textBeginFree,
                                                    const int textEndFree) {
  return alignEndsFree(pattern.c_str(), (int)pattern.length(), patternBeginFree, patternEndFree,
                       text.c_str(), (int)text.length(), textBeginFree, textEndFree);
}
WFAligner::AlignmentStatus WFAligner::alignEndsFree(
    const uint8_t* const pattern, const int patternLength, const int patternBeginFree,
    const int patternEndFree, const uint8_t* const text, const int textLength,
    const int textBeginFree, const int textEndFree) {
  wavefront_aligner_set_alignment_free_ends(wfAligner, patternBeginFree, patternEndFree,
                                            textBeginFree, textEndFree);
  return (AlignmentStatus)wavefront_align_packed2bits(wfAligner, pattern, patternLength, text,
                                                      textLength);
}
WFAligner::AlignmentStatus WFAligner::alignEndsFree(
    int (*matchFunct)(int, int, void*), void* matchFunctArguments, const int patternLength,
    const int patternBeginFree, const int patternEndFree, const int textLength,
    const int textBeginFree, const int textEndFree) {
  wavefront_aligner_set_alignment_free_ends(wfAligner, patternBeginFree, patternEndFree,
                                            textBeginFree, textEndFree);
  return (AlignmentStatus)wavefront_align_lambda(wfAligner, matchFunct, matchFunctArguments,
                                                 patternLength, textLength);
}

// ---------------------------------------------------------------- extension
WFAligner::AlignmentStatus WFAligner::alignExtension(const char* const pattern,
                                                     const int patternLength,
                                                     const char* const text,
                                                     const int textLength) {
  wavefront_aligner_set_alignment_extension(wfAligner);
  return (AlignmentStatus)wavefront_align(wfAligner, pattern, patternLength, text, textLength);
}
WFAligner::AlignmentStatus WFAligner::alignExtension(std::string& pattern, std::string& text) {
  return alignExtension(pattern.c_str(), (int)pattern.length(), text.c_str(),
                        (int)text.length());
}
WFAligner::AlignmentStatus WFAligner::alignExtension(const uint8_t* const pattern,
                                                     const int patternLength,
                                                     const uint8_t* const text,
                                                     const int textLength) {
  wavefront_aligner_set_alignment_extension(wfAligner);
  return (AlignmentStatus)wavefront_align_packed2bits(wfAligner, pattern, patternLength, text,
                                                      textLength);
}
WFAligner::AlignmentStatus WFAligner::alignExtension(int (*matchFunct)(int, int, void*),
                                                     void* matchFunctArguments,
                                                     const int patternLength,
                                                     const int textLength) {
  wavefront_aligner_set_alignment_extension(wfAligner);
  return (AlignmentStatus)wavefront_align_lambda(wfAligner, matchFunct, matchFunctArguments,
                                                 patternLength, textLength);
}

// ---------------------------------------------------------------- batch
int WFAligner::alignBatch(const std::vector<std::string>& patterns,
                          const std::vector<std::string>& texts, std::vector<int>& status,
                          std::vector<int>& score, std::vector<std::string>* cigars) {
  if (patterns.size() != texts.size()) return WF2G_ERR_ARGS;
  const int n = (int)patterns.size();
  std::string seqs;
  std::vector<int64_t> p_off(n), t_off(n), ops_off(n);
  std::vector<int32_t> p_len(n), t_len(n), ops_len(n), st(n), sc(n);
  int64_t ops_total = 0;
  for (int i = 0; i < n; ++i) {
    p_off[i] = (int64_t)seqs.size();
    p_len[i] = (int32_t)patterns[i].size();
    seqs += patterns[i];
    t_off[i] = (int64_t)seqs.size();
    t_len[i] = (int32_t)texts[i].size();
    seqs += texts[i];
    ops_off[i] = ops_total;
    ops_total += (int64_t)p_len[i] + t_len[i];
  }
  const bool alignment = attributes.alignment_scope == compute_alignment;
  std::vector<char> ops(alignment ? (size_t)ops_total + 1 : 1);
  const int rc = wavefront_align_batch(
      wfAligner, n, seqs.data(), p_off.data(), p_len.data(), t_off.data(), t_len.data(),
      sc.data(), st.data(), alignment ? ops.data() : nullptr,
      alignment ? ops_off.data() : nullptr, alignment ? ops_len.data() : nullptr);
  if (rc != WF2G_OK) return rc;
  status.assign(st.begin(), st.end());
  score.assign(sc.begin(), sc.end());
  if (cigars) {
    cigars->assign(n, std::string());
    if (alignment)
      for (int i = 0; i < n; ++i) (*cigars)[i].assign(ops.data() + ops_off[i], ops_len[i]);
  }
  return WF2G_OK;
}

// ---------------------------------------------------------------- heuristics
void WFAligner::setHeuristicNone() { wavefront_aligner_set_heuristic_none(wfAligner); }
void WFAligner::setHeuristicBandedStatic(const int band_min_k, const int band_max_k) {
  wavefront_aligner_set_heuristic_banded_static(wfAligner, band_min_k, band_max_k);
}
void WFAligner::setHeuristicBandedAdaptive(const int band_min_k, const int band_max_k,
                                           const int steps_between_cutoffs) {
  wavefront_aligner_set_heuristic_banded_adaptive(wfAligner, band_min_k, band_max_k,
                                                  steps_between_cutoffs);
}
void WFAligner::setHeuristicWFadaptive(const int min_wavefront_length,
                                       const int max_distance_threshold,
                                       const int steps_between_cutoffs) {
  wavefront_aligner_set_heuristic_wfadaptive(wfAligner, min_wavefront_length,
                                             max_distance_threshold, steps_between_cutoffs);
}
void WFAligner::setHeuristicWFmash(const int min_wavefront_length,
                                   const int max_distance_threshold,
                                   const int steps_between_cutoffs) {
  wavefront_aligner_set_heuristic_wfmash(wfAligner, min_wavefront_length, max_distance_threshold,
                                         steps_between_cutoffs);
}
void WFAligner::setHeuristicXDrop(const int xdrop, const int steps_between_cutoffs) {
  wavefront_aligner_set_heuristic_xdrop(wfAligner, xdrop, steps_between_cutoffs);
}
void WFAligner::setHeuristicZDrop(const int zdrop, const int steps_between_cutoffs) {
  wavefront_aligner_set_heuristic_zdrop(wfAligner, zdrop, steps_between_cutoffs);
}

// ---------------------------------------------------------------- limits
void WFAligner::setMaxAlignmentSteps(const int maxAlignmentSteps) {
  wavefront_aligner_set_max_alignment_steps(wfAligner, maxAlignmentSteps);
}
void WFAligner::setMaxMemory(const uint64_t maxMemoryResident, const uint64_t maxMemoryAbort) {
  wavefront_aligner_set_max_memory(wfAligner, maxMemoryResident, maxMemoryAbort);
}
void WFAligner::setMaxNumThreads(const int maxNumThreads) {
  wavefront_aligner_set_max_num_threads(wfAligner, maxNumThreads);
}

// ---------------------------------------------------------------- accessors
int WFAligner::getAlignmentStatus() { return wfAligner->align_status.status; }
int WFAligner::getAlignmentScore() { return wfAligner->cigar->score; }
void WFAligner::getAlignment(char** const cigarOperations, int* cigarLength) {
  cigar_t* const c = wfAligner->cigar;
  *cigarOperations = c->operations + c->begin_offset;
  *cigarLength = c->end_offset - c->begin_offset;
}
std::string WFAligner::getAlignment() {
  char* ops;
  int len;
  getAlignment(&ops, &len);
  return std::string(ops, (size_t)(len > 0 ? len : 0));
}
void WFAligner::getCIGAR(const bool showMismatches, uint32_t** const cigarOperations,
                         int* const numCigarOperations) {
  cigar_get_CIGAR(wfAligner->cigar, showMismatches, cigarOperations, numCigarOperations);
}
std::string WFAligner::getCIGAR(const bool showMismatches) {
  cigar_t* const c = wfAligner->cigar;
  // at most one run per operation, each at most 11 digits and an op letter
  std::string buf((size_t)(c->end_offset - c->begin_offset) * 12 + 16, '\0');
  const int n = cigar_sprint_SAM_CIGAR(&buf[0], c, showMismatches);
  buf.resize(n > 0 ? (size_t)n : 0);
  return buf;
}

// ---------------------------------------------------------------- display
void WFAligner::printPretty(FILE* const stream, const char* const pattern,
                            const int patternLength, const char* const text,
                            const int textLength) {
  cigar_print_pretty(stream, wfAligner->cigar, pattern, patternLength, text, textLength);
}
char* WFAligner::strStatus(const AlignmentStatus status) {
  return wavefront_align_strerror((int)status);
}
void WFAligner::debugTag(char* const debugTag) {
  wfAligner->align_mode_tag = debugTag;
  if (wfAligner->bialigner != nullptr) {
    wfAligner->bialigner->wf_forward->align_mode_tag = debugTag;
    wfAligner->bialigner->wf_reverse->align_mode_tag = debugTag;
    wfAligner->bialigner->wf_base->align_mode_tag = debugTag;
  }
}

}  // namespace wfa

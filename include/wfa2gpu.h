/*
 * wfa2gpu.h -- C ABI of the GB300 wavefront aligner.
 *
 * Part 1 is the drop-in surface of WFA2-lib's `wavefront_aligner` API: the same
 * type names, field names, enum values and function signatures a C caller of
 * the reference uses, so such a caller recompiles against this header and links
 * libwfa2gpu.so instead of libwfa.a.  Every declaration names the reference
 * interface it replaces (file:line inside smarco/WFA2-lib).
 *
 * Part 2 is the batch surface (no reference counterpart): many pairs per call,
 * with host buffers or device-resident buffers.
 *
 * The alignment itself always runs on the GPU (sm_103a kernels).  There is no
 * CPU fallback: if no usable GPU is present, wavefront_align() returns
 * WF_STATUS_UNATTAINABLE and wavefront_align_batch*() return WF2G_ERR_NO_GPU.
 */
#ifndef WFA2GPU_H_
#define WFA2GPU_H_

#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
/* wavefront/wfa.h:46-55 */
#define WF_STATUS_ALG_COMPLETED            0
#define WF_STATUS_ALG_PARTIAL              1
#define WF_STATUS_MAX_STEPS_REACHED     -100
#define WF_STATUS_OOM                   -200
#define WF_STATUS_UNATTAINABLE          -300
#define WF_STATUS_OK                      -1
#define WF_STATUS_END_REACHED             -2
#define WF_STATUS_END_UNREACHABLE         -3

/* ----------------------------------------------------------------- metrics */
/* wavefront/wavefront_penalties.h:42-48 */
typedef enum {
  indel         = 0,
  edit          = 1,
  gap_linear    = 2,
  gap_affine    = 3,
  gap_affine_2p = 4
} distance_metric_t;

/* alignment/linear_penalties.h:35-40 */
typedef struct {
  int match;
  int mismatch;
  int indel;
} linear_penalties_t;

/* alignment/affine_penalties.h:38-43 */
typedef struct {
  int match;
  int mismatch;
  int gap_opening;
  int gap_extension;
} affine_penalties_t;

/* alignment/affine2p_penalties.h:38-46 */
typedef struct {
  int match;
  int mismatch;
  int gap_opening1;
  int gap_extension1;
  int gap_opening2;
  int gap_extension2;
} affine2p_penalties_t;

/* alignment/affine2p_penalties.h:51-57 */
typedef enum {
  affine2p_matrix_M,
  affine2p_matrix_I1,
  affine2p_matrix_I2,
  affine2p_matrix_D1,
  affine2p_matrix_D2
} affine2p_matrix_type;

/* wavefront/wavefront_penalties.h:53-67 (internal, transformed penalties) */
typedef struct {
  distance_metric_t distance_metric;
  int match;
  int mismatch;
  int gap_opening1;
  int gap_extension1;
  int gap_opening2;
  int gap_extension2;
  linear_penalties_t linear_penalties;
  affine_penalties_t affine_penalties;
  affine2p_penalties_t affine2p_penalties;
  int internal_gap_e;
} wavefront_penalties_t;

/* ------------------------------------------------------------ attributes */
/* wavefront/wavefront_attributes.h:51-66 */
typedef enum {
  compute_score,
  compute_alignment,
} alignment_scope_t;
typedef enum {
  alignment_end2end,
  alignment_endsfree,
} alignment_span_t;
typedef struct {
  alignment_span_t span;
  bool extension;
  int pattern_begin_free;
  int pattern_end_free;
  int text_begin_free;
  int text_end_free;
} alignment_form_t;

/* system/profiler_counter.h:42-51 and system/profiler_timer.h:59-65
 * (kept only so alignment_system_t has the reference's layout) */
typedef struct {
  uint64_t total;
  uint64_t samples;
  uint64_t min;
  uint64_t max;
  double m_oldM;
  double m_newM;
  double m_oldS;
  double m_newS;
} profiler_counter_t;
typedef struct {
  struct timespec begin_timer;
  profiler_counter_t time_ns;
  uint64_t accumulated;
} profiler_timer_t;

/* wavefront/wavefront_attributes.h:71-99 */
typedef struct {
  int max_alignment_steps;
  int probe_interval_global;
  int probe_interval_compact;
  uint64_t max_partial_compacts;
  uint64_t max_memory_compact;
  uint64_t max_memory_resident;
  uint64_t max_memory_abort;
  int verbose;
  bool check_alignment_correct;
  profiler_timer_t timer;
  int max_num_threads;
  int min_offsets_per_thread;
} alignment_system_t;

/* wavefront/wavefront_attributes.h:104-109 */
typedef enum {
  wavefront_memory_high     = 0,
  wavefront_memory_med      = 1,
  wavefront_memory_low      = 2,
  wavefront_memory_ultralow = 3,
} wavefront_memory_t;

/* wavefront/wavefront_heuristic.h:41-69 */
typedef enum {
  wf_heuristic_none            = 0x0000000000000000ul,
  wf_heuristic_banded_static   = 0x0000000000000001ul,
  wf_heuristic_banded_adaptive = 0x0000000000000002ul,
  wf_heuristic_wfadaptive      = 0x0000000000000004ul,
  wf_heuristic_xdrop           = 0x0000000000000010ul,
  wf_heuristic_zdrop           = 0x0000000000000020ul,
  wf_heuristic_wfmash          = 0x0000000000000040ul,
} wf_heuristic_strategy;
typedef struct {
  wf_heuristic_strategy strategy;
  int steps_between_cutoffs;
  int min_k;
  int max_k;
  int min_wavefront_length;
  int max_distance_threshold;
  int xdrop;
  int zdrop;
  int steps_wait;
  int max_sw_score;
  int max_wf_score;
  int max_sw_score_offset;
  int max_sw_score_k;
} wavefront_heuristic_t;

/* wavefront/wavefront_plot.h:45-49 */
typedef struct {
  bool enabled;
  int resolution_points;
  int align_level;
} wavefront_plot_attr_t;

/* system/mm_allocator.h: opaque here; accepted and ignored (device memory is
 * managed by the library's own slab allocator). */
typedef struct _mm_allocator_t mm_allocator_t;

/* wavefront/wavefront_attributes.h:114-133 -- same layout as the reference */
typedef struct {
  distance_metric_t distance_metric;
  alignment_scope_t alignment_scope;
  alignment_form_t alignment_form;
  linear_penalties_t linear_penalties;
  affine_penalties_t affine_penalties;
  affine2p_penalties_t affine2p_penalties;
  wavefront_heuristic_t heuristic;
  wavefront_memory_t memory_mode;
  mm_allocator_t* mm_allocator;
  wavefront_plot_attr_t plot;
  alignment_system_t system;
} wavefront_aligner_attr_t;

/* wavefront/wavefront_attributes.c:38-100 -- same default values */
extern wavefront_aligner_attr_t wavefront_aligner_attr_default;

/* ------------------------------------------------------------------- CIGAR */
/* alignment/cigar.h:45-60 -- same layout as the reference */
typedef struct {
  char* operations;
  int max_operations;
  int begin_offset;
  int end_offset;
  int score;
  int end_v;
  int end_h;
  bool has_misms;
  uint32_t* cigar_buffer;
  int cigar_length;
} cigar_t;

/* ---------------------------------------------------------------- aligner */
typedef struct _wavefront_aligner_t wavefront_aligner_t;

/* wavefront/wfa.h:64-74 */
typedef struct {
  int status;
  int score;
  bool dropped;
  int num_null_steps;
  uint64_t memory_used;
  void (*wf_align_compute)(wavefront_aligner_t* const, const int);
  int (*wf_align_extend)(wavefront_aligner_t* const, const int);
} wavefront_align_status_t;

/* wavefront/wfa.h:79-85 */
typedef enum {
  wf_align_regular = 0,
  wf_align_biwfa = 1,
  wf_align_biwfa_breakpoint_forward = 2,
  wf_align_biwfa_breakpoint_reverse = 3,
  wf_align_biwfa_subsidiary = 4
} wavefront_align_mode_t;

/* The BiWFA sub-aligners (wavefront/wavefront_bialigner.h:43-54), as far as
 * callers touch them (the reference's C++ binding tags their debug mode).
 * The GPU path keeps no host sub-aligners: wavefront_aligner_t.bialigner is
 * always NULL. */
typedef struct {
  wavefront_aligner_t* wf_forward;
  wavefront_aligner_t* wf_reverse;
  wavefront_aligner_t* wf_base;
} wavefront_bialigner_t;

/* wavefront/wfa.h:90-120.  The fields callers read (align_status, cigar,
 * alignment_scope, alignment_form, penalties, heuristic, memory_mode, system,
 * bialigner) keep their names and types; the reference's CPU-only internals
 * (wavefront components, slab, mm_allocator, plot) are replaced by one opaque
 * pointer to the GPU engine. */
typedef struct _wavefront_aligner_t {
  wavefront_align_mode_t align_mode;
  char* align_mode_tag;
  wavefront_align_status_t align_status;
  alignment_scope_t alignment_scope;
  alignment_form_t alignment_form;
  wavefront_penalties_t penalties;
  wavefront_heuristic_t heuristic;
  wavefront_memory_t memory_mode;
  cigar_t* cigar;
  alignment_system_t system;
  wavefront_bialigner_t* bialigner; /* always NULL */
  void* engine; /* GPU engine (device, stream, slab); opaque */
} wavefront_aligner_t;

/* match function of wavefront_align_lambda (alignment/../wavefront_sequences.h:43) */
typedef int (*alignment_match_funct_t)(int, int, void*);

/* -------------------------------------------------------------- functions */
/* wavefront/wfa.h:57-58 */
char* wavefront_align_strerror(const int error_code);
char* wavefront_align_strerror_short(const int error_code);

/* wavefront/wfa.h:125-130 (wavefront/wavefront_aligner.c:422-504) */
wavefront_aligner_t* wavefront_aligner_new(wavefront_aligner_attr_t* attributes);
void wavefront_aligner_reap(wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_delete(wavefront_aligner_t* const wf_aligner);

/* wavefront/wfa.h:135-145 (wavefront/wavefront_aligner.c:508-530).  End-to-end,
 * ends-free and extension forms are computed on the GPU, except two the GPU
 * path does not serve (wavefront_align() then returns WF_STATUS_UNATTAINABLE):
 * ends-free with memory mode ultralow (the reference exits there), and
 * begin-free lengths with match < 0. */
void wavefront_aligner_set_alignment_end_to_end(wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_set_alignment_free_ends(wavefront_aligner_t* const wf_aligner,
    const int pattern_begin_free, const int pattern_end_free,
    const int text_begin_free, const int text_end_free);
void wavefront_aligner_set_alignment_extension(wavefront_aligner_t* const wf_aligner);

/* wavefront/wfa.h:150-180 (wavefront/wavefront_aligner.c:534-604).  Exact
 * alignment needs heuristic none; any other strategy is stored and makes
 * wavefront_align() return WF_STATUS_UNATTAINABLE (the GPU path never
 * silently returns a heuristic, possibly non-optimal, result). */
void wavefront_aligner_set_heuristic_none(wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_set_heuristic_wfadaptive(wavefront_aligner_t* const wf_aligner,
    const int min_wavefront_length, const int max_distance_threshold, const int score_steps);
void wavefront_aligner_set_heuristic_wfmash(wavefront_aligner_t* const wf_aligner,
    const int min_wavefront_length, const int max_distance_threshold, const int score_steps);
void wavefront_aligner_set_heuristic_xdrop(wavefront_aligner_t* const wf_aligner,
    const int xdrop, const int score_steps);
void wavefront_aligner_set_heuristic_zdrop(wavefront_aligner_t* const wf_aligner,
    const int ydrop, const int score_steps);
void wavefront_aligner_set_heuristic_banded_static(wavefront_aligner_t* const wf_aligner,
    const int band_min_k, const int band_max_k);
void wavefront_aligner_set_heuristic_banded_adaptive(wavefront_aligner_t* const wf_aligner,
    const int band_min_k, const int band_max_k, const int score_steps);

/* wavefront/wfa.h:185-194 (wavefront/wavefront_aligner.c:606-645) */
void wavefront_aligner_set_max_alignment_steps(wavefront_aligner_t* const wf_aligner,
    const int max_alignment_steps);
/* wavefront/wavefront_aligner.h:51-66: size, CIGAR trimming and display */
uint64_t wavefront_aligner_get_size(wavefront_aligner_t* const wf_aligner);
bool wavefront_aligner_maxtrim_cigar(wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_print_mode(FILE* const stream, wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_print_scope(FILE* const stream, wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_print_conf(FILE* const stream, wavefront_aligner_t* const wf_aligner);
void wavefront_aligner_set_max_memory(wavefront_aligner_t* const wf_aligner,
    const uint64_t max_memory_resident, const uint64_t max_memory_abort);
void wavefront_aligner_set_max_num_threads(wavefront_aligner_t* const wf_aligner,
    const int max_num_threads);
void wavefront_aligner_set_min_offsets_per_thread(wavefront_aligner_t* const wf_aligner,
    const int min_offsets_per_thread);

/* wavefront/wfa.h:199-204 (wavefront/wavefront_align.c:212-241) */
int wavefront_align(wavefront_aligner_t* const wf_aligner,
    const char* const pattern, const int pattern_length,
    const char* const text, const int text_length);

/* wavefront/wfa.h:205-210.  A host callback cannot run inside a GPU kernel:
 * returns WF_STATUS_UNATTAINABLE. */
int wavefront_align_lambda(wavefront_aligner_t* const wf_aligner,
    alignment_match_funct_t const match_funct, void* match_funct_arguments,
    const int pattern_length, const int text_length);

/* wavefront/wfa.h:211-216.  Sequences packed 4 bases per byte, 2 bits each,
 * first base in the low bits, A=0 C=1 G=2 T=3 (the encoding of
 * wavefront/wavefront_sequences.c:112-136), decoded over all pattern_length
 * bases. */
int wavefront_align_packed2bits(wavefront_aligner_t* const wf_aligner,
    const uint8_t* const pattern, const int pattern_length,
    const uint8_t* const text, const int text_length);

/* alignment/cigar.h:65-160 (alignment/cigar.c) */
cigar_t* cigar_new(const int max_operations);
void cigar_clear(cigar_t* const cigar);
void cigar_resize(cigar_t* const cigar, const int max_operations);
void cigar_free(cigar_t* const cigar);
bool cigar_is_null(const cigar_t* const cigar);
int cigar_count_matches(const cigar_t* const cigar);
void cigar_get_CIGAR(cigar_t* const cigar, const bool show_mismatches,
    uint32_t** const cigar_buffer, int* const cigar_length);
int cigar_score_edit(const cigar_t* const cigar);
int cigar_score_gap_linear(const cigar_t* const cigar, const linear_penalties_t* const penalties);
int cigar_score_gap_affine(const cigar_t* const cigar, const affine_penalties_t* const penalties);
int cigar_score_gap_affine2p(const cigar_t* const cigar, const affine2p_penalties_t* const penalties);
/* alignment/cigar_utils.h:61-69 (maximal-score trimming, cigar_utils.c:112-318) */
bool cigar_maxtrim_gap_linear(cigar_t* const cigar, const linear_penalties_t* const penalties);
bool cigar_maxtrim_gap_affine(cigar_t* const cigar, const affine_penalties_t* const penalties);
bool cigar_maxtrim_gap_affine2p(cigar_t* const cigar, const affine2p_penalties_t* const penalties);
bool cigar_check_alignment(FILE* const stream,
    const char* const pattern, const int pattern_length,
    const char* const text, const int text_length,
    const cigar_t* const cigar, const bool verbose);
void cigar_print(FILE* const stream, const cigar_t* const cigar, const bool print_matches);
int cigar_sprint(char* const buffer, const cigar_t* const cigar, const bool print_matches);
void cigar_print_SAM_CIGAR(FILE* const stream, cigar_t* const cigar, const bool show_mismatches);
int cigar_sprint_SAM_CIGAR(char* const buffer, cigar_t* const cigar, const bool show_mismatches);
void cigar_print_pretty(FILE* const stream, cigar_t* const cigar,
    const char* const pattern, const int pattern_length,
    const char* const text, const int text_length);

/* ================================================================ batch API */
/* No reference counterpart: the reference aligns one pair per call and its
 * benchmark tool loops over pairs with OpenMP
 * (tools/align_benchmark/align_benchmark.c:504-586).  These calls align a whole
 * batch with the same aligner configuration; each pair's result equals what
 * wavefront_align() gives for that pair with that aligner.
 *
 * Layout (host or device, as the call says):
 *   seqs                 concatenated ASCII sequences
 *   pattern_offsets[i]   byte offset of pattern i in seqs   (int64)
 *   pattern_lengths[i]   its length                          (int32)
 *   text_offsets/lengths likewise
 * Outputs:
 *   scores[i]            cigar->score of pair i
 *   status[i]            align_status.status of pair i (WF_STATUS_*)
 *   cigar_ops            operations 'M','X','I','D' (may be NULL in score-only
 *                        mode); pair i writes at cigar_offsets[i] and may use
 *                        up to pattern_lengths[i]+text_lengths[i] bytes
 *   cigar_lengths[i]     number of operations of pair i (may be NULL when
 *                        cigar_ops is NULL)
 * Return: WF2G_OK, or a negative WF2G_ERR_* code for the whole call (per-pair
 * failures are reported in status[]). */
#define WF2G_OK                 0
#define WF2G_ERR_NO_GPU        -1
#define WF2G_ERR_CONFIG        -2
#define WF2G_ERR_ARGS          -3
#define WF2G_ERR_CUDA          -4
#define WF2G_ERR_OOM           -5
/* Per-pair status with no reference counterpart: ends-free lengths longer
 * than the pair's sequences (wavefront_align() prints the reference's
 * message and exits, as wavefront/wavefront_align.c:90-101 does). */
#define WF2G_STATUS_INVALID_FORM -400

int wavefront_align_batch(wavefront_aligner_t* const wf_aligner, const int num_pairs,
    const char* seqs,
    const int64_t* pattern_offsets, const int32_t* pattern_lengths,
    const int64_t* text_offsets, const int32_t* text_lengths,
    int32_t* scores, int32_t* status,
    char* cigar_ops, const int64_t* cigar_offsets, int32_t* cigar_lengths);

/* Same, plus each pair's end position and WFA score: end_info[3i] =
 * cigar->end_v, end_info[3i+1] = cigar->end_h, end_info[3i+2] =
 * align_status.score.  Ends-free alignments end before the sequences' ends;
 * a trimmed extension ends where its CIGAR does ((-1,-1) when it is empty).
 * Not for memory mode ultralow (WF2G_ERR_CONFIG). */
int wavefront_align_batch_ends(wavefront_aligner_t* const wf_aligner, const int num_pairs,
    const char* seqs,
    const int64_t* pattern_offsets, const int32_t* pattern_lengths,
    const int64_t* text_offsets, const int32_t* text_lengths,
    int32_t* scores, int32_t* status,
    char* cigar_ops, const int64_t* cigar_offsets, int32_t* cigar_lengths,
    int32_t* end_info);

/* Same, with every pointer in device memory of the aligner's GPU and the work
 * queued on `cuda_stream` (a cudaStream_t, or NULL for the aligner's own
 * stream).  Returns after the work is queued; synchronise the stream before
 * reading the outputs.  max_sequence_length must bound every pattern and text
 * length in the batch (it sizes the kernels' shared-memory staging). */
int wavefront_align_batch_device(wavefront_aligner_t* const wf_aligner, const int num_pairs,
    const char* d_seqs,
    const int64_t* d_pattern_offsets, const int32_t* d_pattern_lengths,
    const int64_t* d_text_offsets, const int32_t* d_text_lengths,
    const int max_sequence_length,
    int32_t* d_scores, int32_t* d_status,
    char* d_cigar_ops, const int64_t* d_cigar_offsets, int32_t* d_cigar_lengths,
    void* cuda_stream);

/* Allocation-free variant of wavefront_align_batch_device().  No counterpart
 * in the reference.
 *
 * For callers that cannot let a library allocate GPU memory: processes whose
 * device memory belongs to a framework pool or is budgeted to the byte up
 * front (long-running servers, plugins hosted inside another runtime), and
 * code paths where cudaMalloc's implicit device-wide synchronisation cannot be
 * tolerated.  This call never allocates or frees memory and calls no
 * allocating library routine: its scratch (wavefront rows, back-trace bytes,
 * work queue) is one fixed 64 MiB array compiled into the library, which every
 * GPU that loads the library holds until the process exits.  The caller passes
 * inputs and outputs in device memory of the CURRENT device, as for
 * wavefront_align_batch_device(), and the work is queued on `cuda_stream`
 * (NULL: the legacy default stream).  The current device must be the one the
 * aligner was created on, else the call returns WF2G_ERR_ARGS.
 *
 * Limits: memory mode ultralow (BiWFA) is not served (WF2G_ERR_CONFIG); every
 * pattern and text at most 2048 characters (max_sequence_length
 * above that is rejected with WF2G_ERR_ARGS and a message); a pair whose
 * back-trace needs more than 512 KiB of choice bytes reports WF_STATUS_OOM.
 * Concurrency is bounded by the array (tens of warps), so throughput is far
 * below wavefront_align_batch_device().
 *
 * The first call on a device looks up that device's address of the array
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is kept per CUDA context and looked up again when the current
 * context changes (after cudaDeviceReset, for instance), so make the first
 * call after such a reset before any stream capture too.
 * All calls share the array and it keeps the last call's contents (the work
 * queue head is cleared at the start of each call): calls whose GPU work
 * overlaps -- on different streams, or from different threads -- race on it
 * and must be serialised by the caller. */
int wavefront_align_batch_device_noalloc(wavefront_aligner_t* const wf_aligner,
    const int num_pairs, const char* d_seqs,
    const int64_t* d_pattern_offsets, const int32_t* d_pattern_lengths,
    const int64_t* d_text_offsets, const int32_t* d_text_lengths,
    const int max_sequence_length,
    int32_t* d_scores, int32_t* d_status,
    char* d_cigar_ops, const int64_t* d_cigar_offsets, int32_t* d_cigar_lengths,
    void* cuda_stream);

/* Kernel launches issued by this aligner since it was created (an audit
 * counter for benchmarks). */
int64_t wavefront_aligner_gpu_launches(const wavefront_aligner_t* const wf_aligner);

/* CUDA device the library uses (the current device at wavefront_aligner_new()),
 * or -1 when no usable GPU is present. */
int wfa2gpu_device(void);

/* ------------------------------------------------------------------ serving
 * Continuous batching of single-pair requests on one GPU (no counterpart in
 * the reference, whose callers loop over wavefront_align()).  Requests are
 * queued by wavefront_server_submit() from any thread; worker lanes admit
 * what has arrived into batches within the device-memory budget and run them
 * concurrently on the GPU; a pair whose back-trace exceeds the per-warp
 * budget is re-run in BiWFA mode (wavefront_memory_ultralow), and its result
 * says so.  Each result equals what wavefront_align() returns for that pair
 * with the aligner's configuration (memory mode high) or, for BiWFA re-runs,
 * with memory mode ultralow. */
typedef struct wavefront_server_t wavefront_server_t;

typedef struct {
  int64_t hbm_budget_bytes; /* device memory the server may use; 0: 80 GiB */
  int64_t backtrace_budget_bytes; /* back-trace bytes of one pair before it is
                                     re-run in BiWFA mode; 0: 64 MiB */
  int lanes;                /* batches in flight on the GPU; 0: 2 */
  int max_batch_pairs;      /* pairs per batch; 0: 65536 */
  int batch_window_us;      /* wait for more requests before a batch; <0: 200 */
  int biwfa_min_length;     /* admission: pairs this long (pattern or text) are
                               predicted over budget and aligned in BiWFA mode
                               directly; 0: 8192, <0: never */
} wavefront_server_attr_t;

typedef struct {
  int64_t id;             /* as returned by wavefront_server_submit() */
  int status;             /* WF_STATUS_* */
  int score;              /* cigar->score */
  int memory_mode;        /* wavefront_memory_high, or _ultralow for BiWFA re-runs */
  const char* operations; /* CIGAR operations (M/X/I/D), valid until the next poll */
  int operations_length;
  double latency_us;      /* submit to result */
} wavefront_server_result_t;

/* Server with the configuration of `wf_aligner` (end-to-end, heuristic none,
 * memory mode high; score-only or full CIGAR).  NULL if that configuration is
 * not served or no GPU is present. */
wavefront_server_t* wavefront_server_new(const wavefront_aligner_t* const wf_aligner,
                                         const wavefront_server_attr_t* const attributes);
/* Queues one pair (copied); returns its id (>= 0) or a WF2G_ERR_* code. */
int64_t wavefront_server_submit(wavefront_server_t* const server, const char* const pattern,
                                const int pattern_length, const char* const text,
                                const int text_length);
/* Up to max_results finished results, waiting up to timeout_us for the first;
 * returns their number (0 if none finished in time). */
int wavefront_server_poll(wavefront_server_t* const server, wavefront_server_result_t* results,
                          const int max_results, const int timeout_us);
/* Requests submitted and not yet returned by wavefront_server_poll(). */
int64_t wavefront_server_in_flight(wavefront_server_t* const server);
/* Kernel launches issued by the server so far. */
int64_t wavefront_server_gpu_launches(wavefront_server_t* const server);
/* Finishes the queued work, stops the lanes and frees the server. */
void wavefront_server_delete(wavefront_server_t* const server);

#ifdef __cplusplus
}
#endif
#endif /* WFA2GPU_H_ */

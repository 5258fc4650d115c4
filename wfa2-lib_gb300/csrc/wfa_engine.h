/*
 * wfa_engine.h -- internal C interface between the host C layer
 * (wfa_aligner.c) and the CUDA engine (wfa_engine.cu).  Not installed.
 */
#ifndef WFA2GPU_ENGINE_H_
#define WFA2GPU_ENGINE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Alignment configuration after the reference's penalty set-up
 * (wavefront/wavefront_penalties.c:95-173): x/o/e are the internal
 * (possibly Eizenga-transformed) penalties, match the user's match (<=0). */
typedef struct {
  int metric; /* 3 gap_affine, 4 gap_affine_2p */
  int match;
  int x, o1, e1, o2, e2;
  int score_only;
  int max_steps; /* INT32_MAX when unlimited */
  int ultralow;  /* 1: BiWFA (wavefront_memory_ultralow) */
  /* heuristic strategy: a bit set of wf_heuristic_strategy values
   * (wavefront/wavefront_heuristic.h:41-49), 0 exact, and its parameters */
  int heur, h_min_len, h_max_dist, h_steps;
  int h_xdrop, h_zdrop, h_min_k, h_max_k;
  /* alignment form (wavefront/wavefront_attributes.h:55-69): endsfree = 1
   * with the four free lengths, or extension = 1 (per-pair presets and
   * maximal-score trimming with the user's penalties um..ue2) */
  int endsfree, extension, pbf, pef, tbf, tef;
  int um, ux, uo1, ue1, uo2, ue2;
} wf2g_cfg_t;

/* Creates an engine on the current CUDA device; NULL (and *err set to a
 * WF2G_ERR_* code) if no usable GPU is present. */
void* wf2g_engine_new(int* err);
void wf2g_engine_free(void* engine);

/* Aligns a batch.  on_device=0: every pointer is host memory, the call copies
 * in, computes and copies out, and returns when the results are in place.
 * on_device=1: every pointer is device memory, work is queued on `stream`
 * (NULL: the engine's own stream) and the call returns without waiting.
 * max_len bounds the pattern and text lengths (computed when on_device=0).
 * end_info (optional, 3 int32 per pair): cigar->end_v, cigar->end_h and the
 * WFA score (align_status.score). */
int wf2g_engine_align(void* engine, const wf2g_cfg_t* cfg, int num_pairs, int on_device,
                      const char* seqs, const int64_t* p_off, const int32_t* p_len,
                      const int64_t* t_off, const int32_t* t_len, int max_len,
                      int32_t* scores, int32_t* status, char* ops, const int64_t* ops_off,
                      int32_t* ops_len, int32_t* end_info, void* stream);

int64_t wf2g_engine_launches(const void* engine);

/* Device and pinned host bytes the engine holds (its buffers grow on demand
 * and are kept for the next call). */
int64_t wf2g_engine_bytes(const void* engine);

/* Allocation-free batch alignment on the current device (wfa_noalloc.cu):
 * device pointers only, scratch from a fixed array in the library image. */
int wf2g_noalloc_align(const wf2g_cfg_t* cfg, int num_pairs, const char* d_seqs,
                       const int64_t* d_p_off, const int32_t* d_p_len, const int64_t* d_t_off,
                       const int32_t* d_t_len, int max_len, int32_t* d_scores, int32_t* d_status,
                       char* d_ops, const int64_t* d_ops_off, int32_t* d_ops_len, void* stream);
int wf2g_engine_device(void);
/* The device an engine was created on. */
int wf2g_engine_owner_device(const void* engine);

/* Serving loop (wfa_server.cu); the result type is wavefront_server_result_t
 * of include/wfa2gpu.h, passed as void* to keep this header self-contained. */
void* wf2g_server_new(const wf2g_cfg_t* cfg, int64_t hbm_budget, int64_t backtrace_budget,
                      int lanes, int max_batch, int window_us, int biwfa_min_length, int* err);
int64_t wf2g_server_submit(void* srv, const char* pattern, int plen, const char* text, int tlen);
int wf2g_server_poll(void* srv, void* results, int max, int timeout_us);
int64_t wf2g_server_in_flight(void* srv);
int64_t wf2g_server_launches(void* srv);
void wf2g_server_free(void* srv);

#ifdef __cplusplus
}
#endif
#endif /* WFA2GPU_ENGINE_H_ */

/*
 * wfa_bench_loop.c -- benchmark helper: the plain per-pair drop-in usage.
 *
 * A C caller of WFA2-lib aligns a batch by calling wavefront_align() once per
 * pair (tools/align_benchmark/align_benchmark.c:452-503).  This loop does
 * exactly that against libwfa2gpu.so, so the per-pair GPU path is timed
 * without any interpreter overhead.
 */
#define _POSIX_C_SOURCE 200112L
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <time.h>

#include "wfa2gpu.h"

double wf2g_bench_per_pair(wavefront_aligner_t* wf, int n, const char* seqs,
                           const int64_t* p_off, const int32_t* p_len, const int64_t* t_off,
                           const int32_t* t_len, int32_t* scores, int32_t* status,
                           int32_t* ops_len) {
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  for (int i = 0; i < n; ++i) {
    status[i] = wavefront_align(wf, seqs + p_off[i], p_len[i], seqs + t_off[i], t_len[i]);
    scores[i] = wf->cigar->score;
    ops_len[i] = wf->cigar->end_offset - wf->cigar->begin_offset;
  }
  clock_gettime(CLOCK_MONOTONIC, &b);
  return (double)(b.tv_sec - a.tv_sec) + 1e-9 * (double)(b.tv_nsec - a.tv_nsec);
}

/* ------------------------------------------------------------ serving load
 * Open-loop load generator for the serving loop: a submitter thread submits
 * pair i at arrival_us[i] (microseconds after the start), the calling thread
 * polls results until all n have returned.  Request ids of this run start at
 * id_base (the number of requests the server accepted before).  Per pair: latency (submit to
 * result, measured by the server), status, score, memory mode and CRC-32 of
 * the CIGAR operations.  Returns the wall time from the start to the last
 * result (seconds), or a negative value on error. */
static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static uint32_t crc32_bytes(const char* p, int n) {
  uint32_t c = 0xFFFFFFFFu;
  for (int i = 0; i < n; ++i) {
    c ^= (uint8_t)p[i];
    for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
  }
  return c ^ 0xFFFFFFFFu;
}

typedef struct {
  wavefront_server_t* srv;
  int n;
  const char* seqs;
  const int64_t *p_off, *t_off;
  const int32_t *p_len, *t_len;
  const double* arrival_us;
  double t0;
  int64_t* ids;
  int failed;
} submit_job_t;

static void* submitter(void* arg) {
  submit_job_t* j = (submit_job_t*)arg;
  for (int i = 0; i < j->n; ++i) {
    const double due = j->t0 + 1e-6 * j->arrival_us[i];
    for (;;) {
      const double now = now_s();
      if (now >= due) break;
      const double wait = due - now;
      if (wait > 200e-6) {
        struct timespec ts;
        ts.tv_sec = 0;
        ts.tv_nsec = (long)((wait - 100e-6) * 1e9);
        nanosleep(&ts, NULL);
      }
    }
    j->ids[i] = wavefront_server_submit(j->srv, j->seqs + j->p_off[i], j->p_len[i],
                                        j->seqs + j->t_off[i], j->t_len[i]);
    if (j->ids[i] < 0) j->failed = 1;
  }
  return NULL;
}

double wf2g_bench_serve(wavefront_server_t* srv, int64_t id_base, int n, const char* seqs,
                        const int64_t* p_off,
                        const int32_t* p_len, const int64_t* t_off, const int32_t* t_len,
                        const double* arrival_us, double* latency_us, int32_t* status,
                        int32_t* scores, int32_t* modes, uint32_t* cigar_crc) {
  if (n <= 0) return 0.0;
  int64_t* ids = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  wavefront_server_result_t* res = (wavefront_server_result_t*)malloc(sizeof(*res) * 4096);
  if (!ids || !res) return -1.0;
  submit_job_t job = {srv, n, seqs, p_off, t_off, p_len, t_len, arrival_us, now_s(), ids, 0};
  pthread_t th;
  if (pthread_create(&th, NULL, submitter, &job) != 0) return -1.0;
  int got = 0;
  double t_last = job.t0;
  while (got < n) {
    const int k = wavefront_server_poll(srv, res, 4096, 1000);
    if (k < 0) break;
    for (int r = 0; r < k; ++r) {
      const int64_t i = res[r].id - id_base;
      if (i < 0 || i >= n) continue;
      latency_us[i] = res[r].latency_us;
      status[i] = res[r].status;
      scores[i] = res[r].score;
      modes[i] = res[r].memory_mode;
      cigar_crc[i] = crc32_bytes(res[r].operations, res[r].operations_length);
      ++got;
    }
    if (k > 0) t_last = now_s();
    if (job.failed) break;
  }
  pthread_join(th, NULL);
  free(ids);
  free(res);
  if (job.failed || got < n) return -2.0;
  return t_last - job.t0;
}

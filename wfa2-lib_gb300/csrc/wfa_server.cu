// wfa_server.cu -- serving loop: continuous batching of single-pair requests
// on one GPU.
//
//   submit   copies the pair into host memory and queues it (any thread)
//   queues   requests are binned by predicted cost (the longer sequence):
//            short (< 2048), medium (< biwfa_min_length), and long pairs,
//            which are predicted over the back-trace budget and go to BiWFA
//   lanes    worker threads, each with its own engine (CUDA stream, device
//            buffers and wavefront scratch: its share of the HBM budget),
//            assigned to the short and medium queues in turn.  A lane takes
//            what is queued (up to its pair and byte limits, after waiting at
//            most the batch window for more), aligns it through the batch
//            path and publishes the results.  While one lane's batch is on
//            the GPU the others admit the requests that arrived meanwhile, so
//            batches overlap on the device, and short pairs never wait behind
//            long ones.
//   fallback long pairs, and pairs whose back-trace does not fit the per-warp
//            cap (WF_STATUS_OOM from the last pass), are aligned in BiWFA mode
//            (ultralow memory) by a dedicated lane; their results say so.
//   poll     returns finished results with their submit-to-finish latency.
//
// Device memory is allocated by the engines on first use and reused: after
// warm-up the loop runs without cudaMalloc.  Results are identical to the
// batch path on the same pairs (alone or mixed): every pair is aligned
// independently by the same kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "wfa2gpu.h"
#include "wfa_engine_impl.cuh"

namespace wf2g {
namespace eng {
namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  int64_t id;
  std::string P, T;
  Clock::time_point t_submit;
};

struct Res {
  int64_t id;
  int32_t status, score, mode;
  std::string ops;
  double latency_us;
};

struct PinnedBuf {
  void* p = nullptr;
  size_t cap = 0;
  bool ensure(size_t bytes) {
    if (bytes <= cap) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    const size_t want = bytes + bytes / 4 + 4096;
    if (cudaMallocHost(&p, want) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    cap = want;
    return true;
  }
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace

struct Server {
  wf2g_cfg_t cfg;
  int device = 0;
  int max_batch = 65536;
  int64_t max_batch_bytes = 256ll << 20;
  int window_us = 200;
  std::vector<void*> engines;  // lanes, then the fallback lane
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_fb, cv_done;
  std::deque<Req> queue[2], fallback;  // short / medium pairs; BiWFA pairs
  int nlanes = 0;
  static constexpr int kShortLen = 2048;
  std::deque<Res> done;
  std::vector<Res> polled;  // kept alive until the next poll
  int64_t next_id = 0;
  int64_t in_flight = 0;
  bool stop = false;
  int biwfa_min_length = 8192;  // < 0: never direct

  int lanes_alive = 0;

  void publish(std::vector<Res>& rs) {
    std::lock_guard<std::mutex> g(mu);
    for (Res& r : rs) done.push_back(std::move(r));
    cv_done.notify_all();
  }
  // called with mu held
  void in_flight_polled(size_t n) { in_flight -= (int64_t)n; }

  // Aligns `batch` on engine E with configuration c; fills per-request
  // status/score/ops.  Pairs are grouped by length so that the wavefront
  // scratch of each launch is sized for its own pairs.
  void run_batch(void* E, const wf2g_cfg_t& c, std::vector<Req>& batch, std::vector<int32_t>& st,
                 std::vector<int32_t>& sc, std::vector<std::string>& ops, PinnedBuf& hbuf) {
    const int n = (int)batch.size();
    st.assign(n, kStUnattainable);
    sc.assign(n, 0);
    ops.assign(n, std::string());
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto len = [&](int i) { return std::max(batch[i].P.size(), batch[i].T.size()); };
    std::sort(order.begin(), order.end(), [&](int a, int b) { return len(a) < len(b); });
    const size_t bounds[3] = {2048, 16384, SIZE_MAX};
    int j0 = 0;
    for (int b = 0; b < 3 && j0 < n; ++b) {
      int j1 = j0;
      while (j1 < n && len(order[j1]) <= bounds[b]) ++j1;
      if (j1 == j0) continue;
      const int m = j1 - j0;
      int64_t seq = 0, opsz = 0;
      for (int j = j0; j < j1; ++j) {
        seq += (int64_t)batch[order[j]].P.size() + batch[order[j]].T.size();
        opsz += (int64_t)batch[order[j]].P.size() + batch[order[j]].T.size();
      }
      // pinned layout: seqs | p_off | p_len | t_off | t_len | scores | status | ops_off | ops_len | ops
      const size_t need = (size_t)seq + 16 + (size_t)m * (8 + 4 + 8 + 4 + 4 + 4 + 8 + 4) + 64 +
                          (size_t)opsz + 16;
      if (!hbuf.ensure(need)) {
        j0 = j1;
        continue;  // leaves kStUnattainable
      }
      char* base = (char*)hbuf.p;
      char* seqs = base;
      size_t o = ((size_t)seq + 16 + 7) & ~size_t(7);
      int64_t* p_off = (int64_t*)(base + o); o += (size_t)m * 8;
      int64_t* t_off = (int64_t*)(base + o); o += (size_t)m * 8;
      int64_t* ops_off = (int64_t*)(base + o); o += (size_t)m * 8;
      int32_t* p_len = (int32_t*)(base + o); o += (size_t)m * 4;
      int32_t* t_len = (int32_t*)(base + o); o += (size_t)m * 4;
      int32_t* scores = (int32_t*)(base + o); o += (size_t)m * 4;
      int32_t* status = (int32_t*)(base + o); o += (size_t)m * 4;
      int32_t* ops_len = (int32_t*)(base + o); o += (size_t)m * 4;
      char* opsb = base + ((o + 15) & ~size_t(15));
      int64_t at = 0, ot = 0;
      for (int j = 0; j < m; ++j) {
        const Req& r = batch[order[j0 + j]];
        p_off[j] = at;
        p_len[j] = (int32_t)r.P.size();
        memcpy(seqs + at, r.P.data(), r.P.size());
        at += (int64_t)r.P.size();
        t_off[j] = at;
        t_len[j] = (int32_t)r.T.size();
        memcpy(seqs + at, r.T.data(), r.T.size());
        at += (int64_t)r.T.size();
        ops_off[j] = ot;
        ot += (int64_t)r.P.size() + r.T.size();
      }
      const bool cig = !c.score_only;
      const int rc = wf2g_engine_align(E, &c, m, 0, seqs, p_off, p_len, t_off, t_len, 0, scores,
                                       status, cig ? opsb : nullptr, cig ? ops_off : nullptr,
                                       cig ? ops_len : nullptr, nullptr, nullptr);
      for (int j = 0; j < m; ++j) {
        const int i = order[j0 + j];
        if (rc != 0) {
          st[i] = rc == WF2G_ERR_OOM_ ? kStOOM : kStUnattainable;
          continue;
        }
        st[i] = status[j];
        sc[i] = scores[j];
        if (cig && status[j] == kStCompleted) ops[i].assign(opsb + ops_off[j], (size_t)ops_len[j]);
      }
      j0 = j1;
    }
  }

  void lane_main(int lane) {
    cudaSetDevice(device);
    void* E = engines[lane];
    PinnedBuf hbuf;
    std::vector<Req> batch;
    std::vector<int32_t> st, sc;
    std::vector<std::string> ops;
    // queues this lane serves, in order of preference
    const int mine = nlanes >= 2 ? lane % 2 : -1;
    auto pick = [&]() -> std::deque<Req>* {
      if (mine >= 0) return queue[mine].empty() ? nullptr : &queue[mine];
      if (!queue[0].empty()) return &queue[0];
      return queue[1].empty() ? nullptr : &queue[1];
    };
    while (true) {
      batch.clear();
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || pick() != nullptr; });
        std::deque<Req>* q = pick();
        if (stop && !q) {
          if (--lanes_alive == 0) cv_fb.notify_all();
          return;
        }
        // batch window: let more requests arrive while the queue is short
        if ((int)q->size() < max_batch && window_us > 0) {
          cv_work.wait_for(lk, std::chrono::microseconds(window_us),
                           [&] { return stop || (int)q->size() >= max_batch; });
        }
        int64_t bytes = 0;
        while (!q->empty() && (int)batch.size() < max_batch) {
          const int64_t b = (int64_t)q->front().P.size() + q->front().T.size();
          if (!batch.empty() && bytes + b > max_batch_bytes) break;
          bytes += b;
          batch.push_back(std::move(q->front()));
          q->pop_front();
        }
        if (!q->empty()) cv_work.notify_all();
      }
      run_batch(E, cfg, batch, st, sc, ops, hbuf);
      std::vector<Res> out;
      std::vector<Req> over;
      const auto now = Clock::now();
      for (size_t i = 0; i < batch.size(); ++i) {
        if (st[i] == kStOOM && !cfg.score_only) {
          over.push_back(std::move(batch[i]));
          continue;
        }
        out.push_back(Res{batch[i].id, st[i], sc[i], 0, std::move(ops[i]),
                          std::chrono::duration<double, std::micro>(now - batch[i].t_submit).count()});
      }
      if (!over.empty()) {
        std::lock_guard<std::mutex> g(mu);
        for (Req& r : over) fallback.push_back(std::move(r));
        cv_fb.notify_one();
      }
      if (!out.empty()) publish(out);
    }
  }

  void fallback_main() {
    cudaSetDevice(device);
    void* E = engines.back();
    wf2g_cfg_t c = cfg;
    c.ultralow = 1;
    PinnedBuf hbuf;
    std::vector<Req> batch;
    std::vector<int32_t> st, sc;
    std::vector<std::string> ops;
    while (true) {
      batch.clear();
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_fb.wait(lk, [&] { return (stop && lanes_alive == 0) || !fallback.empty(); });
        if (stop && lanes_alive == 0 && fallback.empty()) return;
        while (!fallback.empty() && (int)batch.size() < max_batch) {
          batch.push_back(std::move(fallback.front()));
          fallback.pop_front();
        }
      }
      run_batch(E, c, batch, st, sc, ops, hbuf);
      std::vector<Res> out;
      const auto now = Clock::now();
      for (size_t i = 0; i < batch.size(); ++i)
        out.push_back(Res{batch[i].id, st[i], sc[i], 3, std::move(ops[i]),
                          std::chrono::duration<double, std::micro>(now - batch[i].t_submit).count()});
      publish(out);
    }
  }
};

}  // namespace eng
}  // namespace wf2g

using wf2g::eng::Server;

extern "C" void* wf2g_server_new(const wf2g_cfg_t* cfg, int64_t hbm_budget,
                                 int64_t backtrace_budget, int lanes, int max_batch,
                                 int window_us, int biwfa_min_length, int* err) {
  using namespace wf2g::eng;
  const int dev = wf2g_engine_device();
  if (dev < 0) {
    if (err) *err = WF2G_ERR_NO_GPU_;
    return nullptr;
  }
  // the BiWFA fallback has no ends-free form (wavefront/wavefront_align.c:67-82)
  // and serves the gap-affine metrics only
  if (!cfg || cfg->ultralow || cfg->endsfree || cfg->metric <= 2 || (cfg->heur & ~wf2g::kHsWfadaptive)) {
    if (err) *err = WF2G_ERR_CONFIG_;
    return nullptr;
  }
  Server* S = new (std::nothrow) Server();
  if (!S) {
    if (err) *err = WF2G_ERR_OOM_;
    return nullptr;
  }
  S->cfg = *cfg;
  S->device = dev;
  S->biwfa_min_length = biwfa_min_length;
  if (max_batch > 0) S->max_batch = max_batch;
  if (window_us >= 0) S->window_us = window_us;
  if (lanes <= 0) lanes = 2;
  if (hbm_budget <= 0) hbm_budget = 80ll << 30;
  // budget split: each lane's wavefront scratch and batch buffers, and the
  // BiWFA lane's rows and buffers
  const int64_t share = hbm_budget / (lanes + 1);
  for (int l = 0; l <= lanes; ++l) {
    int e = 0;
    void* E = wf2g_engine_new(&e);
    if (!E) {
      for (void* x : S->engines) wf2g_engine_free(x);
      delete S;
      if (err) *err = e;
      return nullptr;
    }
    Engine* en = (Engine*)E;
    en->scratch_budget = share / 2;
    en->bi_scratch_budget = share / 4;
    en->pool_budget = share / 4;
    // back-trace bytes a pair may use: pairs needing more are over budget
    // and go to BiWFA
    en->bits_cap = backtrace_budget > 0 ? backtrace_budget : 64ll << 20;
    S->engines.push_back(E);
  }
  S->max_batch_bytes = std::max<int64_t>(1 << 20, share / 64);
  S->lanes_alive = lanes;
  S->nlanes = lanes;
  for (int l = 0; l < lanes; ++l) S->threads.emplace_back(&Server::lane_main, S, l);
  S->threads.emplace_back(&Server::fallback_main, S);
  if (err) *err = WF2G_OK_;
  return S;
}

extern "C" int64_t wf2g_server_submit(void* srv, const char* pattern, int plen, const char* text,
                                      int tlen) {
  Server* S = (Server*)srv;
  if (!S || plen < 0 || tlen < 0 || (plen && !pattern) || (tlen && !text)) return WF2G_ERR_ARGS_;
  wf2g::eng::Req r;
  r.P.assign(pattern ? pattern : "", (size_t)plen);
  r.T.assign(text ? text : "", (size_t)tlen);
  r.t_submit = wf2g::eng::Clock::now();
  // admission: long pairs are predicted over the back-trace budget and go to
  // the BiWFA lane at once (full CIGAR only; score-only runs keep no back-trace)
  const bool direct = !S->cfg.score_only && S->biwfa_min_length > 0 &&
                      std::max(plen, tlen) >= S->biwfa_min_length;
  std::lock_guard<std::mutex> g(S->mu);
  r.id = S->next_id++;
  const int64_t id = r.id;
  S->in_flight++;
  if (direct) {
    S->fallback.push_back(std::move(r));
    S->cv_fb.notify_one();
  } else {
    S->queue[std::max(plen, tlen) < Server::kShortLen ? 0 : 1].push_back(std::move(r));
    S->cv_work.notify_all();
  }
  return id;
}

// Copies up to max finished results; waits up to timeout_us for the first.
extern "C" int wf2g_server_poll(void* srv, void* results, int max, int timeout_us) {
  Server* S = (Server*)srv;
  if (!S || max < 0 || (max > 0 && !results)) return WF2G_ERR_ARGS_;
  wavefront_server_result_t* out = (wavefront_server_result_t*)results;
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->done.empty() && timeout_us > 0)
    S->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !S->done.empty(); });
  S->polled.clear();
  while (!S->done.empty() && (int)S->polled.size() < max) {
    S->polled.push_back(std::move(S->done.front()));
    S->done.pop_front();
  }
  for (size_t i = 0; i < S->polled.size(); ++i) {
    const wf2g::eng::Res& r = S->polled[i];
    out[i].id = r.id;
    out[i].status = r.status;
    out[i].score = r.score;
    out[i].memory_mode = r.mode;
    out[i].operations = r.ops.data();
    out[i].operations_length = (int)r.ops.size();
    out[i].latency_us = r.latency_us;
  }
  S->in_flight_polled(S->polled.size());
  return (int)S->polled.size();
}

extern "C" int64_t wf2g_server_in_flight(void* srv) {
  Server* S = (Server*)srv;
  if (!S) return 0;
  std::lock_guard<std::mutex> g(S->mu);
  return S->in_flight;
}

extern "C" int64_t wf2g_server_launches(void* srv) {
  Server* S = (Server*)srv;
  if (!S) return 0;
  int64_t n = 0;
  for (void* E : S->engines) n += wf2g_engine_launches(E);
  return n;
}

extern "C" void wf2g_server_free(void* srv) {
  Server* S = (Server*)srv;
  if (!S) return;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
    S->cv_fb.notify_all();
  }
  for (std::thread& t : S->threads) t.join();
  for (void* E : S->engines) wf2g_engine_free(E);
  delete S;
}

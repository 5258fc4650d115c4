#!/usr/bin/env python3
"""Benchmark of the GB300 wavefront aligner (one JSON line on rank 0).

Workload (default): 1,000,000 synthetic gap-affine (4,6,2) pairs per GPU,
|P| ~ U[500,1500], divergence ~ U[0,15%], full CIGAR, end-to-end, memory
mode high -- the batched configuration the headline metric is quoted on.
One step = one batched alignment of all pairs of this rank.

value   pairs/s with inputs resident in HBM (kernels only, CUDA events on the
        launching stream); inputs (~2 GB) exceed the 126 MB L2 between steps
e2e     pairs/s through the public host API wavefront_align_batch(): per step
        the H2D copy of the inputs from pinned memory and the D2H copy of the
        results (scores, status, CIGAR operations) are inside the timed region
--impl reference   the CPU implementation of the path on the host cores
        (oracle/_ref when the reference was built here, else the C restatement
        in oracle/), on a bounded sample of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wfa2-lib_gb300"))

METRIC = "pairs/s bit-exact score+CIGAR, batched vs per-pair on 1 GB300; p50/p99 latency"
INT_OPS_PER_CELL = {3: 20, 4: 25}  # int32 ops per WFA cell: gap-affine, gap-affine-2p
INT_OPS_PER_EXT_WORD = 8   # per additional 32-base extend word
MEM_HIGH, MEM_ULTRALOW = 0, 3
# DRAM bytes (read + write) per pair of the dominant kernel, from one ncu
# capture of a 20,000-pair launch of the first fast pass on the headline
# workload (dram__bytes_read.sum + dram__bytes_write.sum = 0.1806 + 0.7180 GB;
# profiles/wfa_fast2_kernel_workload1.md), scaled to a launch by its pairs
TRAFFIC_BYTES_PER_PAIR = {(1, False): 898.60e6 / 20000}

# The benchmark configurations: workload of the seeded generator, pairs per
# GPU, distance metric, memory mode, pairs of the per-pair drop-in sample and
# first size of the CPU sample.
CONFIGS = {
    0: dict(workload=0, pairs=10_000, metric=3, memory=MEM_HIGH, per_pair=2000, cpu_n=1000,
            name="100bp, 5% single-base edits"),
    1: dict(workload=1, pairs=1_000_000, metric=3, memory=MEM_HIGH, per_pair=2000, cpu_n=1000,
            name="500-1500bp, 0-15% divergence, 10% geometric indels"),
    2: dict(workload=2, pairs=50_000, metric=4, memory=MEM_HIGH, per_pair=200, cpu_n=64,
            name="1-10kbp log-uniform, 5% divergence, 20% long indels, affine2p (4,6,2,24,1)"),
    3: dict(workload=3, pairs=1000, metric=3, memory=MEM_ULTRALOW, per_pair=4, cpu_n=16,
            name="100kbp, 10-15% divergence, BiWFA (ultralow memory)"),
    4: dict(workload=4, pairs=50_000, metric=3, memory=MEM_HIGH, per_pair=0, cpu_n=200,
            name="serving: Poisson arrivals at 200k pairs/s, lognormal length (median 2kbp, "
                 "100bp-50kbp), 1-20% divergence, 80 GB budget, BiWFA fallback"),
}
SERVE_RATE = 200_000.0  # offered load of the serving configuration (pairs/s)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=sorted(CONFIGS),
                    help="benchmark configuration (1: the headline batched workload)")
    ap.add_argument("--pairs", type=int, default=0, help="pairs per GPU (0: the config's)")
    ap.add_argument("--score-only", action="store_true")
    ap.add_argument("--per-pair-sample", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=8.0,
                    help="target wall time of the bounded CPU-baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serve-sweep", action="store_true",
                    help="config 4: skip the latency-against-load sweep")
    ap.add_argument("--fixed", default="",
                    help="L:D -- instead of the config's pairs, pairs of fixed length L with "
                         "D per-mille uniform edits (generator workload 5; small profiling cases)")
    a = ap.parse_args()
    c = CONFIGS[a.config]
    a.workload = c["workload"]
    a.param = a.param2 = 0
    if a.fixed:
        a.workload = 5
        a.param, a.param2 = (int(x) for x in a.fixed.split(":"))
    a.metric = c["metric"]
    a.memory = c["memory"]
    a.pairs = a.pairs or c["pairs"]
    a.per_pair_sample = a.per_pair_sample or c["per_pair"]
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _timed_device(torch, stream, step, steps):
    """CUDA-event time of `steps` calls of step() on `stream` after one untimed call."""
    step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0


def secondary_lines(W, O, torch, args, stream, d_seqs, d_poff, d_plen, d_toff, d_tlen, max_len,
                    d_scores, d_status, d_ops, d_opsoff, d_opslen, p, n):
    """Bounded measurements of the other configurations inside the headline
    run, so that each has a recorded number: the headline batch under the
    library's default heuristic (wf-adaptive 10,50,1), a sample of config 2
    (affine2p, 1-10 kbp) and of config 3 (BiWFA, 100 kbp), each with a
    parity check."""
    out = {}
    dev = d_seqs.device
    # -- config 1 with wf-adaptive (10,50,1), full CIGAR, the same device batch
    wa = W.Aligner(W.Config(wfadaptive=(10, 50, 1)))

    def step_wa():
        rc = wa.align_batch_device(n, d_seqs.data_ptr(), d_poff.data_ptr(), d_plen.data_ptr(),
                                   d_toff.data_ptr(), d_tlen.data_ptr(), max_len,
                                   d_scores.data_ptr(), d_status.data_ptr(), d_ops.data_ptr(),
                                   d_opsoff.data_ptr(), d_opslen.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"wf-adaptive batch failed: {rc}")
    wa_s = _timed_device(torch, stream, step_wa, args.steps)
    wa.close()
    k = min(n, 20000)
    g_sc, g_st = d_scores[:k].cpu().numpy(), d_status[:k].cpu().numpy()
    g_len = d_opslen[:k].cpu().numpy()
    offs = d_opsoff[:k + 1].cpu().numpy()
    g_ops = d_ops[:int(offs[-1])].cpu().numpy()
    b = O.PairBatch(p.seqs, p.p_off[:k], p.p_len[:k], p.t_off[:k], p.t_len[:k])
    r = O.align(b, O.Penalties(), wfadaptive=(10, 50, 1), nthreads=os.cpu_count() or 1)
    flagged = (r.flags & O.FLAG_STALE_SOURCE) != 0
    bad = 0
    for i in np.flatnonzero(~flagged):
        cig = g_ops[offs[i]:offs[i] + g_len[i]].tobytes().decode()
        bad += (int(g_sc[i]) != int(r.score[i])) or (int(g_st[i]) != int(r.status[i])) or \
            (cig != r.cigar(i))
    assert bad == 0, f"wf-adaptive parity: {bad} mismatches"
    out["config1_wfadaptive"] = {
        "value": n * args.steps / wa_s, "unit": "pairs/s", "ms_per_step": 1000 * wa_s / args.steps,
        "parity": f"first {k} pairs: scores, statuses and CIGARs equal the checker's "
                  f"({int(flagged.sum())} flagged stale-source pairs skipped)"}

    # -- config 2 sample: affine2p (4,6,2,24,1), 1-10 kbp, full CIGAR
    q = W.generate(2, 2000, first=0)
    ql = q.p_len.astype(np.int64) + q.t_len
    qo = np.zeros(q.n + 1, np.int64)
    np.cumsum(ql, out=qo[1:])
    t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev)
         for x in (q.seqs, q.p_off, q.p_len, q.t_off, q.t_len, qo)]
    qs, qst = (torch.empty(q.n, dtype=torch.int32, device=dev) for _ in range(2))
    qops = torch.empty(int(qo[-1]) + 16, dtype=torch.uint8, device=dev)
    qol = torch.empty(q.n, dtype=torch.int32, device=dev)
    a2 = W.Aligner(W.Config(metric=4))
    qmax = int(max(q.p_len.max(), q.t_len.max()))

    def step_a2():
        rc = a2.align_batch_device(q.n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                                   t[3].data_ptr(), t[4].data_ptr(), qmax, qs.data_ptr(),
                                   qst.data_ptr(), qops.data_ptr(), t[5].data_ptr(),
                                   qol.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"affine2p batch failed: {rc}")
    a2_s = _timed_device(torch, stream, step_a2, 1)
    a2.close()
    kk = 8
    b2 = O.PairBatch(q.seqs, q.p_off[:kk], q.p_len[:kk], q.t_off[:kk], q.t_len[:kk])
    r2 = O.align(b2, O.Penalties(metric=4), nthreads=os.cpu_count() or 1)
    g2 = qs[:kk].cpu().numpy()
    assert np.array_equal(g2, r2.score) and (qst[:kk].cpu().numpy() == 0).all(), "affine2p parity"
    out["config2_affine2p_sample"] = {
        "value": q.n / a2_s, "unit": "pairs/s",
        "sample": f"{q.n} pairs of the config-2 workload, device-resident, one step",
        "parity": f"first {kk} scores equal the checker's"}

    # -- config 3 sample: BiWFA (ultralow memory), 100 kbp, full CIGAR; its
    # scores against the unidirectional score-only run of the same pairs
    z = W.generate(3, 48, first=0)
    zl = z.p_len.astype(np.int64) + z.t_len
    zo = np.zeros(z.n + 1, np.int64)
    np.cumsum(zl, out=zo[1:])
    u = [torch.from_numpy(np.ascontiguousarray(x)).to(dev)
         for x in (z.seqs, z.p_off, z.p_len, z.t_off, z.t_len, zo)]
    zs, zst = (torch.empty(z.n, dtype=torch.int32, device=dev) for _ in range(2))
    zops = torch.empty(int(zo[-1]) + 16, dtype=torch.uint8, device=dev)
    zol = torch.empty(z.n, dtype=torch.int32, device=dev)
    zmax = int(max(z.p_len.max(), z.t_len.max()))
    bi = W.Aligner(W.Config(memory_mode=MEM_ULTRALOW))

    def step_bi():
        rc = bi.align_batch_device(z.n, u[0].data_ptr(), u[1].data_ptr(), u[2].data_ptr(),
                                   u[3].data_ptr(), u[4].data_ptr(), zmax, zs.data_ptr(),
                                   zst.data_ptr(), zops.data_ptr(), u[5].data_ptr(),
                                   zol.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"BiWFA batch failed: {rc}")
    bi_s = _timed_device(torch, stream, step_bi, 1)
    bi.close()
    bi_scores = zs.cpu().numpy().copy()
    uni = W.Aligner(W.Config(score_only=True))
    rc = uni.align_batch_device(z.n, u[0].data_ptr(), u[1].data_ptr(), u[2].data_ptr(),
                                u[3].data_ptr(), u[4].data_ptr(), zmax, zs.data_ptr(),
                                zst.data_ptr(), 0, 0, 0, stream.cuda_stream)
    torch.cuda.synchronize()
    uni.close()
    assert rc == 0 and np.array_equal(bi_scores, zs.cpu().numpy()), "BiWFA score parity"
    out["config3_biwfa_sample"] = {
        "value": z.n / bi_s, "unit": "pairs/s",
        "sample": f"{z.n} pairs of the config-3 workload (100 kbp), device-resident, one step "
                  "(a batch this small is bound by the longest pair's latency)",
        "parity": "BiWFA scores equal the unidirectional score-only scores"}
    return out


def gen_pinned(W, torch, workload, n, first, param=0, param2=0):
    """Seeded pairs in pinned host memory."""
    def alloc(nbytes):
        return torch.empty(nbytes, dtype=torch.uint8, pin_memory=True).numpy()
    p = W.generate(workload, n, first=first, param=param, param2=param2, alloc=alloc)

    def pin(a):
        t = torch.empty(a.shape, dtype={np.int64: torch.int64, np.int32: torch.int32}[a.dtype.type],
                        pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()
    return W.Pairs(p.seqs, pin(p.p_off), pin(p.p_len), pin(p.t_off), pin(p.t_len))


def cpu_sample(O, W, args, target_s, first, kind):
    """Times the CPU path on a bounded sample; returns (pairs/s, sample n, threads, res)."""
    threads = os.cpu_count() or 1
    pen = O.Penalties(metric=args.metric)
    n = CONFIGS[args.config]["cpu_n"]
    while True:
        p = W.generate(args.workload, n, first=first, param=args.param, param2=args.param2)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        t0 = time.perf_counter()
        r = O.align(b, pen, memory_mode=args.memory, score_only=args.score_only, kind=kind,
                    nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= target_s * 0.5 or n >= 200_000:
            return n / dt, n, threads, r, p, dt
        n = min(200_000, int(n * max(2.0, target_s / max(dt, 1e-3))))


def run_reference(args, rank):
    """--impl reference: the CPU implementation on the host cores."""
    if rank != 0:
        return
    import wfa2gpu as W
    from oracle import oracle as O
    W.build() if not os.path.exists(W.GEN_PATH) else None
    O.build(ref=False)
    kind = "reference" if O.have_reference() else "port"
    vals = []
    for _ in range(args.warmup):
        cpu_sample(O, W, args, 1.0, 0, kind)
    for _ in range(args.steps):
        v, n, threads, _, _, dt = cpu_sample(O, W, args, args.cpu_seconds / max(args.steps, 1),
                                             0, kind)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * n / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": kind,
                         "sample": f"{n} pairs of the workload per step"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    c = CONFIGS[args.config]
    pen = "gap-affine-2p(0,4,6,2,24,1)" if args.metric == 4 else "gap-affine(0,4,6,2)"
    mem = "ultralow (BiWFA)" if args.memory == MEM_ULTRALOW else "high"
    name = c["name"]
    if args.fixed:
        name = f"fixed length {args.param}, {args.param2 / 10:g}% uniform edits"
    return {"workload": f"config {args.config}: batched {pen} end-to-end "
                        f"{'score-only' if args.score_only else 'full CIGAR'}, memory {mem}, "
                        f"{args.pairs} pairs/GPU of workload {args.workload} ({name})",
            "pairs_per_gpu": args.pairs, "seq": "uint8 ASCII ACGT",
            "l2": "inputs larger than L2 (126 MB) at the default sizes; no flush needed",
            "parallelism": f"replicas x{args.gpus} (pairs sharded, no collective)"}


def run_serving(args, rank, world, local):
    """Config 4: the serving loop under open-loop Poisson arrivals.

    One step = n requests submitted at their arrival times by a native
    submitter thread (libwfa2bench.so) and polled until all have returned.
    value = requests completed per second over the step; latency = submit to
    result, per request.  The same pairs are also aligned offline in one
    batch (wavefront_align_batch) for comparison, and every served result is
    checked against the batch path in the memory mode the server used."""
    import torch
    import zlib
    import wfa2gpu as W
    from oracle import oracle as O
    torch.cuda.set_device(local)
    if not os.path.exists(W.LIB_PATH):
        W.build()
    n = args.pairs
    first = rank * n
    p = W.generate(args.workload, n, first=first)
    rng = np.random.default_rng(1234 + rank)
    arrivals = np.cumsum(rng.exponential(1e6 / SERVE_RATE, n)).astype(np.float64)
    cfg = W.Config()
    srv = W.Server(cfg, hbm_budget_bytes=80 << 30, lanes=2)
    bl = C.CDLL(os.path.join(W.PKG_DIR, "lib", "libwfa2bench.so"))
    P = C.c_void_p
    bl.wf2g_bench_serve.restype = C.c_double
    bl.wf2g_bench_serve.argtypes = [P, C.c_int64, C.c_int] + [P] * 11

    def ptr(a):
        return C.c_void_p(a.ctypes.data)
    lat = np.zeros(n, np.float64)
    st = np.zeros(n, np.int32)
    sc = np.zeros(n, np.int32)
    md = np.zeros(n, np.int32)
    crc = np.zeros(n, np.uint32)
    submitted = 0

    def serve(m, arr):
        nonlocal submitted
        wall = bl.wf2g_bench_serve(C.c_void_p(srv._h), submitted, m, ptr(p.seqs), ptr(p.p_off),
                                   ptr(p.p_len), ptr(p.t_off), ptr(p.t_len), ptr(arr), ptr(lat),
                                   ptr(st), ptr(sc), ptr(md), ptr(crc))
        submitted += m
        if wall < 0:
            raise RuntimeError(f"serving run failed ({wall})")
        return wall
    # warm-up: short runs at the same rate (engines size their buffers)
    wm = min(n, 5000)
    for _ in range(max(args.warmup, 3)):
        serve(wm, np.ascontiguousarray(arrivals[:wm] - arrivals[0]))
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    l0 = srv.launches
    walls, lats = [], []
    for _ in range(args.steps):
        walls.append(serve(n, arrivals))
        lats.append(lat.copy())
        assert (st == 0).all(), f"{int((st != 0).sum())} requests failed"
    launches = srv.launches - l0
    clk = clocks.stop()
    wall = statistics.median(walls)
    value = n / wall
    L = np.concatenate(lats) / 1000.0
    # Latency against load: the offered rate above is far beyond what the GPU
    # completes, so its latencies are the queue's drain time.  Here Poisson
    # streams at fractions of the completed rate just measured, each about
    # six seconds long (at least 2,000 requests).
    sweep = []
    if not args.no_serve_sweep:
        srng = np.random.default_rng(4321 + rank)
        for frac in (0.25, 0.5, 0.8, 1.0):
            rate = frac * value
            m = int(min(n, max(2000, rate * 6.0)))
            arr = np.ascontiguousarray(np.cumsum(srng.exponential(1e6 / rate, m)))
            w = serve(m, arr)
            assert (st[:m] == 0).all(), f"{int((st[:m] != 0).sum())} requests failed"
            Lm = lat[:m] / 1000.0
            sweep.append({"offered_fraction_of_capacity": frac, "offered_rate": rate,
                          "requests": m, "completed_pairs_per_s": m / w,
                          "latency_ms": {"p50": float(np.percentile(Lm, 50)),
                                         "p99": float(np.percentile(Lm, 99)),
                                         "max": float(Lm.max())}})
        # the last sweep run overwrote the first m results: the parity check
        # below needs the main run's, so serve the main stream once more
        serve(n, arrivals)
    srv.close()
    # offline batched form on the same pairs (host API, all pairs in one call)
    al = W.Aligner(cfg)
    al.align_batch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    t0 = time.perf_counter()
    rc, b_sc, b_st, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len, p.t_off,
                                                          p.t_len)
    t_batch = time.perf_counter() - t0
    al.close()
    # parity of the last step: high-mode results against the batch path, BiWFA
    # re-runs against the ultralow batch path
    hi = md == MEM_HIGH
    b_crc = np.array([zlib.crc32(ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes())
                      for i in range(n)], np.uint32)
    assert np.array_equal(sc[hi], b_sc[hi]) and np.array_equal(crc[hi], b_crc[hi])
    fb = np.nonzero(~hi)[0]
    if len(fb):
        ul = W.Aligner(W.Config(memory_mode=MEM_ULTRALOW))
        sub = W.Pairs(p.seqs, np.ascontiguousarray(p.p_off[fb]), np.ascontiguousarray(p.p_len[fb]),
                      np.ascontiguousarray(p.t_off[fb]), np.ascontiguousarray(p.t_len[fb]))
        rc2, u_sc, u_st, uops, uol, uoo = ul.align_batch(sub.seqs, sub.p_off, sub.p_len,
                                                         sub.t_off, sub.t_len)
        ul.close()
        u_crc = np.array([zlib.crc32(uops[uoo[j]:uoo[j] + uol[j]].tobytes())
                          for j in range(len(fb))], np.uint32)
        assert np.array_equal(sc[fb], u_sc) and np.array_equal(crc[fb], u_crc)
    if rank != 0:
        return
    cpu_v, cpu_n, cpu_threads, _, _, _ = cpu_sample(O, W, args, args.cpu_seconds, 0, "port")
    seq_bytes = int(np.sum(p.p_len) + np.sum(p.t_len))
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * wall,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded SplitMix64 generator; seeded Poisson arrivals)",
        "config": workload_config(args),
        "serving": {"offered_rate": SERVE_RATE, "requests_per_step": n,
                    "latency_ms": {"p50": float(np.percentile(L, 50)),
                                   "p99": float(np.percentile(L, 99)),
                                   "max": float(L.max())},
                    "note": "offered 200k pairs/s is beyond capacity: these latencies are "
                            "queue drain; see sweep for latency at sustainable load",
                    "sweep": sweep,
                    "biwfa_fallback_pairs": int(len(fb)),
                    "offline_batched_pairs_per_s": n / t_batch,
                    "lanes": 2, "hbm_budget_gb": 80},
        "roofline": None,
        "cpu_baseline": {"value": cpu_v, "unit": "pairs/s", "cores": cpu_threads, "kind": "port",
                         "sample": f"first {cpu_n} pairs of the workload, all host threads"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": seq_bytes,
                "d2h_bytes_per_step": int(n * 8 + np.sum(ops_len))},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.config == 4:
        run_serving(args, rank, world, local)
        return
    import torch
    import wfa2gpu as W
    from oracle import oracle as O

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0 or not os.path.exists(W.LIB_PATH):
        W.build() if not os.path.exists(W.LIB_PATH) else None
    if dist:
        dist.barrier()

    # ------------------------------------------------------------ data
    n = args.pairs
    first = rank * n
    p = gen_pinned(W, torch, args.workload, n, first, args.param, args.param2)
    max_len = p.max_len
    cigar = not args.score_only
    cap = p.p_len.astype(np.int64) + p.t_len.astype(np.int64)
    ops_off = np.zeros(n + 1, np.int64)
    np.cumsum(cap, out=ops_off[1:])

    dev = torch.device("cuda", local)
    seq_bytes = int(p.t_off[-1] + p.t_len[-1])
    d_seqs = torch.from_numpy(p.seqs).to(dev)
    d_poff = torch.from_numpy(p.p_off).to(dev)
    d_plen = torch.from_numpy(p.p_len).to(dev)
    d_toff = torch.from_numpy(p.t_off).to(dev)
    d_tlen = torch.from_numpy(p.t_len).to(dev)
    d_scores = torch.empty(n, dtype=torch.int32, device=dev)
    d_status = torch.empty(n, dtype=torch.int32, device=dev)
    d_ops = torch.empty(int(ops_off[-1]) + 16 if cigar else 16, dtype=torch.uint8, device=dev)
    d_opsoff = torch.from_numpy(ops_off).to(dev)
    d_opslen = torch.empty(n, dtype=torch.int32, device=dev)

    cfg = W.Config(metric=args.metric, score_only=args.score_only, memory_mode=args.memory)
    al = W.Aligner(cfg)
    # a non-default stream: the C ABI maps a NULL stream to the aligner's own
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def step_device():
        rc = al.align_batch_device(
            n, d_seqs.data_ptr(), d_poff.data_ptr(), d_plen.data_ptr(), d_toff.data_ptr(),
            d_tlen.data_ptr(), max_len, d_scores.data_ptr(), d_status.data_ptr(),
            d_ops.data_ptr() if cigar else 0, d_opsoff.data_ptr() if cigar else 0,
            d_opslen.data_ptr() if cigar else 0, stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"wavefront_align_batch_device failed: {rc}")

    for _ in range(max(args.warmup, 3)):
        step_device()
    torch.cuda.synchronize()
    status = d_status.cpu().numpy()
    if not (status == 0).all():
        raise RuntimeError(f"{int((status != 0).sum())} pairs did not complete")

    # ------------------------------------------------------------ timed (device-resident)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = al.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = al.launches - l0
    clk = clocks.stop()
    dev_s = ev0.elapsed_time(ev1) / 1000.0
    if dist:
        t = torch.tensor([dev_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    value = world * n * args.steps / dev_s

    # ------------------------------------------------------------ e2e (host API)
    e2e = None
    if not args.no_e2e:
        h_scores = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
        h_status = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
        h_ops = torch.empty(int(ops_off[-1]) + 16 if cigar else 16, dtype=torch.uint8,
                            pin_memory=True).numpy()
        h_opslen = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy()
        h_opsoff = torch.empty(n + 1, dtype=torch.int64, pin_memory=True).numpy()
        h_opsoff[...] = ops_off

        # the host API as a caller uses it: its own aligner, host buffers in,
        # host buffers out
        al_h = W.Aligner(cfg)

        def step_host():
            rc = al_h.align_batch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len,
                                ops_off=h_opsoff if cigar else None, scores=h_scores,
                                status=h_status, ops=h_ops if cigar else None,
                                ops_len=h_opslen if cigar else None)[0]
            if rc != 0:
                raise RuntimeError(f"wavefront_align_batch failed: {rc}")
        step_host()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_host()
        e2e_s = time.perf_counter() - t0
        al_h.close()
        if dist:
            t = torch.tensor([e2e_s], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        h2d = seq_bytes + n * (8 + 4 + 8 + 4) + (n * 8 if cigar else 0)
        d2h = n * 8 + ((n * 4 + int(ops_off[-1])) if cigar else 0)
        e2e = {"value": world * n * args.steps / e2e_s, "unit": "pairs/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    # ------------------------------------------------------------ parity
    # The timed batch's results, every pair: scores, statuses and CIGARs
    # against the CPU checker, every CIGAR replayed and rescored
    # (oracle/wfa_check.c).  The checker's run over the whole batch, with all
    # host threads, is also the CPU baseline and gives the exact work units.
    pen = O.Penalties(metric=args.metric)
    g_scores, g_status = d_scores.cpu().numpy(), d_status.cpu().numpy()
    g_ops = d_ops.cpu().numpy() if cigar else None
    g_opslen = d_opslen.cpu().numpy() if cigar else None
    full_check = args.config in (0, 1)
    threads = os.cpu_count() or 1
    parity, r_full, cpu_full_s = None, None, None
    if full_check:
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        r_full = O.align(b, pen, memory_mode=args.memory, score_only=args.score_only,
                         nthreads=threads)
        cpu_full_s = time.perf_counter() - t0
        parity = O.compare(b, pen, g_scores, g_status, g_ops, ops_off[:n], g_opslen, r_full,
                           score_only=args.score_only, nthreads=threads)
        if e2e is not None:
            # the host-API results equal the device-resident ones, pair by pair
            pe = O.compare(b, pen, h_scores, h_status, h_ops, ops_off[:n], h_opslen,
                           O.AlignResult(g_scores, g_status, g_ops, ops_off[:n], g_opslen,
                                         None, None),
                           score_only=args.score_only, nthreads=threads)
            parity["e2e_vs_device_mismatch"] = (pe["score_mismatch"] + pe["status_mismatch"] +
                                                pe["cigar_mismatch"])
        counts = [parity[k] for k in ("score_mismatch", "status_mismatch", "cigar_mismatch",
                                      "cigar_invalid", "rescore_mismatch")]
        counts.append(parity.get("e2e_vs_device_mismatch", 0))
        if dist:
            t = torch.tensor(counts + [n], dtype=torch.int64, device=dev)
            dist.all_reduce(t)
            counts, checked = t.tolist()[:-1], int(t.tolist()[-1])
            parity.update(dict(zip(("score_mismatch", "status_mismatch", "cigar_mismatch",
                                    "cigar_invalid", "rescore_mismatch"), counts[:5])))
            parity["pairs_checked"] = checked
        parity["checker"] = "oracle port (C restatement), all pairs of the timed batch"
        if any(counts):
            print(json.dumps({"parity_failed": parity}), flush=True)
            raise SystemExit(f"parity failure: {parity}")
    elif e2e is not None:
        assert np.array_equal(h_scores, g_scores)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ------------------------------------------------------------ rank-0 extras
    # per-pair drop-in: wavefront_align() once per pair from C
    bl = C.CDLL(os.path.join(W.PKG_DIR, "lib", "libwfa2bench.so"))
    bl.wf2g_bench_per_pair.restype = C.c_double
    P = C.c_void_p
    bl.wf2g_bench_per_pair.argtypes = [P, C.c_int, P, P, P, P, P, P, P, P]
    k = max(1, min(args.per_pair_sample, n))
    ps, pst, pl = (np.zeros(k, np.int32) for _ in range(3))

    def ptr(a):
        return C.c_void_p(a.ctypes.data)
    pa = W.Aligner(cfg)
    bl.wf2g_bench_per_pair(C.cast(pa._h, P), min(k, 50), ptr(p.seqs), ptr(p.p_off),
                           ptr(p.p_len), ptr(p.t_off), ptr(p.t_len), ptr(ps), ptr(pst), ptr(pl))
    per_pair_s = bl.wf2g_bench_per_pair(C.cast(pa._h, P), k, ptr(p.seqs), ptr(p.p_off),
                                        ptr(p.p_len), ptr(p.t_off), ptr(p.t_len), ptr(ps),
                                        ptr(pst), ptr(pl))
    pa.close()
    per_pair = k / per_pair_s
    assert np.array_equal(ps, d_scores[:k].cpu().numpy())

    # Secondary lines of the headline run (cheap, same box, same process):
    # the drop-in on the configuration the reference names for it (100 bp
    # pairs), and the headline batch score-only (checked against the
    # checker's scores of the full run).
    secondary = {}
    if args.config == 1 and not args.fixed and not args.score_only:
        p0 = W.generate(0, 2000, first=0)
        r0 = O.align(O.PairBatch(p0.seqs, p0.p_off, p0.p_len, p0.t_off, p0.t_len),
                     O.Penalties(), nthreads=os.cpu_count() or 1)
        k0 = p0.n
        s0, t0s, l0s = (np.zeros(k0, np.int32) for _ in range(3))
        pa0 = W.Aligner(cfg)
        bl.wf2g_bench_per_pair(C.cast(pa0._h, P), 100, ptr(p0.seqs), ptr(p0.p_off), ptr(p0.p_len),
                               ptr(p0.t_off), ptr(p0.t_len), ptr(s0), ptr(t0s), ptr(l0s))
        w0 = bl.wf2g_bench_per_pair(C.cast(pa0._h, P), k0, ptr(p0.seqs), ptr(p0.p_off),
                                    ptr(p0.p_len), ptr(p0.t_off), ptr(p0.t_len), ptr(s0), ptr(t0s),
                                    ptr(l0s))
        pa0.close()
        assert np.array_equal(s0, r0.score) and (t0s == 0).all(), "config 0 drop-in parity"
        secondary["config0_per_pair_dropin"] = {
            "value": k0 / w0, "unit": "pairs/s",
            "sample": f"{k0} wavefront_align() calls on 100 bp pairs (5 edits each), "
                      "scores checked against the checker"}
        so = W.Aligner(W.Config(metric=args.metric, score_only=True, memory_mode=args.memory))

        def step_score_only():
            rc = so.align_batch_device(n, d_seqs.data_ptr(), d_poff.data_ptr(), d_plen.data_ptr(),
                                       d_toff.data_ptr(), d_tlen.data_ptr(), max_len,
                                       d_scores.data_ptr(), d_status.data_ptr(), 0, 0, 0,
                                       stream.cuda_stream)
            if rc != 0:
                raise RuntimeError(f"score-only batch failed: {rc}")
        for _ in range(max(args.warmup, 3)):
            step_score_only()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step_score_only()
        e1.record(stream)
        torch.cuda.synchronize()
        so.close()
        so_s = e0.elapsed_time(e1) / 1000.0
        so_scores = d_scores.cpu().numpy()
        so_ok = bool(r_full is not None and np.array_equal(so_scores, r_full.score) and
                     (d_status.cpu().numpy() == 0).all())
        assert so_ok, "score-only parity"
        secondary["config1_score_only"] = {
            "value": n * args.steps / so_s, "unit": "pairs/s", "ms_per_step": 1000 * so_s / args.steps,
            "parity": f"all {n} scores equal the checker's"}
        secondary.update(secondary_lines(W, O, torch, args, stream, d_seqs, d_poff, d_plen, d_toff,
                                         d_tlen, max_len, d_scores, d_status, d_ops, d_opsoff,
                                         d_opslen, p, n))

    # CPU baseline and work units (WFA cells, extend chars): the checker's run
    # over the whole batch where it ran, else a bounded sample of the workload
    if r_full is not None and world == 1:
        r, cpu_n, cpu_threads = r_full, n, threads
        cpu_v = n / cpu_full_s
        cpu_desc = f"all {n} pairs of the timed batch, all host threads (also the parity check)"
    else:
        cpu_v, cpu_n, cpu_threads, r, sp, _ = cpu_sample(O, W, args, args.cpu_seconds, 0, "port")
        cpu_desc = f"first {cpu_n} pairs of the workload, all host threads"
        if r_full is not None:
            r = r_full
        # the bounded sample is a parity check of the timed results' first pairs
        if parity is None and first == 0:
            m = min(cpu_n, n)
            sb = O.PairBatch(p.seqs, p.p_off[:m], p.p_len[:m], p.t_off[:m], p.t_len[:m])
            ref = O.AlignResult(r.score[:m], r.status[:m], r.ops, r.ops_off[:m], r.ops_len[:m],
                                None, None)
            parity = O.compare(sb, pen, g_scores[:m], g_status[:m], g_ops, ops_off[:m],
                               g_opslen[:m] if cigar else None, ref,
                               score_only=args.score_only, nthreads=cpu_threads)
            parity["checker"] = "oracle port (C restatement), the bounded CPU sample"
            bad = sum(parity[k] for k in ("score_mismatch", "status_mismatch", "cigar_mismatch",
                                          "cigar_invalid", "rescore_mismatch"))
            if bad:
                print(json.dumps({"parity_failed": parity}), flush=True)
                raise SystemExit(f"parity failure: {parity}")
    unit_note = "WFA cells of the exact unidirectional reference (heuristic none)"
    if args.memory == MEM_ULTRALOW:
        # BiWFA's work is counted in the unidirectional unit, so its extra
        # (forward, reverse and base-case) cells count against the fraction:
        # the same sample, score-only, memory high, for the cell count only
        ub = O.PairBatch(sp.seqs, sp.p_off, sp.p_len, sp.t_off, sp.t_len)
        r = O.align(ub, pen, memory_mode=MEM_HIGH, score_only=True, nthreads=cpu_threads)
        unit_note += " (BiWFA's own cells count as overhead)"
    cells_pp = float(r.cells.mean())
    ext_words_pp = float(np.ceil(r.ext / 32.0).mean())
    ops_pp = INT_OPS_PER_CELL[args.metric] * cells_pp + INT_OPS_PER_EXT_WORD * ext_words_pp
    step_s = dev_s / args.steps
    sm_mhz = clk.get("sm_mhz") or 2070.0
    num_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    peak_tops = num_sms * 128 * sm_mhz * 1e6 / 1e12
    achieved_tops = n * ops_pp / step_s / 1e12
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    alg_bytes = seq_bytes + n * 4 + (int(np.sum(pl)) * n / k if cigar else 0)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * step_s,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded SplitMix64 generator)", "config": workload_config(args),
        "roofline": {"bound": "int32", "achieved": achieved_tops, "peak": peak_tops,
                     "unit": "Tops/s", "frac": achieved_tops / peak_tops,
                     "traffic": (TRAFFIC_BYTES_PER_PAIR[(args.config, args.score_only)] * n
                                 if (args.config, args.score_only) in TRAFFIC_BYTES_PER_PAIR
                                 and not args.fixed else None),
                     "traffic_basis": "DRAM read+write bytes per launch of the first fast pass, "
                                      "ncu capture of 20,000 pairs scaled by pairs",
                     "work_unit": unit_note,
                     "units_per_launch": {"wfa_cells": n * cells_pp,
                                          "ops_per_cell": INT_OPS_PER_CELL[args.metric],
                                          "ext_words": n * ext_words_pp},
                     "peak_basis": f"{num_sms} SMs x 128 int32 lanes x {sm_mhz:.0f} MHz "
                                   "(median SM clock sampled during the run)",
                     "hbm": {"achieved_gbs": alg_bytes / step_s / 1e9, "peak_gbs": hbm_peak,
                             "frac": alg_bytes / step_s / 1e9 / hbm_peak,
                             "peak_basis": "MEASURED_PEAKS.json hbm_gbs (of measured)"}},
        "cpu_baseline": {"value": cpu_v, "unit": "pairs/s", "cores": cpu_threads, "kind": "port",
                         "sample": cpu_desc},
        "e2e": e2e,
        "parity": parity,
        "gpu_launches": launches,
        "clocks": clk,
        "per_pair_dropin": {"value": per_pair, "unit": "pairs/s",
                            "sample": f"{k} wavefront_align() calls"},
        "secondary": secondary,
        "batched_over_per_pair": value / world / per_pair,
        "cells_per_s": world * n * cells_pp * args.steps / dev_s,
        "dp_cell_updates_per_s": float(np.sum(p.p_len.astype(np.float64) * p.t_len)) * world *
        args.steps / dev_s,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

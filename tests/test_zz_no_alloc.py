"""wavefront_align_batch_device_noalloc(): the entry point for callers that
cannot let the library allocate GPU memory (their device memory belongs to a
framework pool or a fixed budget, or cudaMalloc's device-wide synchronisation
is not acceptable on their path).  Its scratch is a fixed array inside the
library, shared by every call.

Checked through the C ABI against wavefront_align_batch_device() on the same
inputs, on two calls in a row (the second call reuses the array the first one
left behind).  Integer results: equality is exact.  This file is collected last
so that a failure here does not stop the rest of the suite."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WF2G_ERR_ARGS = -3


def _device_batch(torch, W, p):
    dev = torch.device("cuda", 0)
    n = p.n
    cap = p.p_len.astype(np.int64) + p.t_len.astype(np.int64)
    ops_off = np.zeros(n + 1, np.int64)
    np.cumsum(cap, out=ops_off[1:])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = dict(seqs=T(p.seqs), poff=T(p.p_off), plen=T(p.p_len), toff=T(p.t_off),
             tlen=T(p.t_len), opsoff=T(ops_off))
    return d, ops_off


def _outputs(torch, n, total_ops):
    dev = torch.device("cuda", 0)
    return dict(scores=torch.full((n,), -7, dtype=torch.int32, device=dev),
                status=torch.full((n,), -7, dtype=torch.int32, device=dev),
                ops_len=torch.full((n,), -7, dtype=torch.int32, device=dev),
                ops=torch.zeros(total_ops + 16, dtype=torch.uint8, device=dev))


def _run(al, noalloc, n, d, o, max_len, score_only, stream):
    fn = al.align_batch_device_noalloc if noalloc else al.align_batch_device
    return fn(n, d["seqs"].data_ptr(), d["poff"].data_ptr(), d["plen"].data_ptr(),
              d["toff"].data_ptr(), d["tlen"].data_ptr(), max_len, o["scores"].data_ptr(),
              o["status"].data_ptr(), 0 if score_only else o["ops"].data_ptr(),
              0 if score_only else d["opsoff"].data_ptr(),
              0 if score_only else o["ops_len"].data_ptr(), stream)


def _host(o, ops_off, n, score_only):
    scores = o["scores"].cpu().numpy()
    status = o["status"].cpu().numpy()
    if score_only:
        return scores, status, None
    ops = o["ops"].cpu().numpy()
    ol = o["ops_len"].cpu().numpy()
    cig = [ops[ops_off[i]:ops_off[i] + ol[i]].tobytes() for i in range(n)]
    return scores, status, cig


# (label, configuration keywords, generator workload): the exact gap-affine
# default, gap-affine-2p and the wf-adaptive heuristic -- the kernel choices
# this entry point serves.  Gap-affine-2p runs on 100 bp pairs: on 1 kbp pairs
# its back-trace can pass the 512 KiB per warp (a documented OOM).
CONFIGS = [("affine", {}, 1), ("affine2p", {"metric": 4}, 0),
           ("wfadaptive", {"wfadaptive": (10, 50, 1)}, 1)]


@pytest.mark.parametrize("score_only", [False, True])
@pytest.mark.parametrize("label,kw,workload", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_noalloc_matches_batch_device_twice(score_only, label, kw, workload):
    torch = pytest.importorskip("torch")
    import wfa2gpu as W
    W.build()
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    p = W.generate(workload, 600 if label == "affine" else 200, first=4242)
    assert p.max_len <= 2048
    n = p.n
    d, ops_off = _device_batch(torch, W, p)
    stream = torch.cuda.Stream()
    al = W.Aligner(W.Config(score_only=score_only, **kw))

    ref = _outputs(torch, n, int(ops_off[-1]))
    assert _run(al, False, n, d, ref, p.max_len, score_only, stream.cuda_stream) == 0
    torch.cuda.synchronize()
    exp = _host(ref, ops_off, n, score_only)
    assert (exp[1] == 0).all()

    for call in range(2):
        out = _outputs(torch, n, int(ops_off[-1]))
        rc = _run(al, True, n, d, out, p.max_len, score_only, stream.cuda_stream)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        got = _host(out, ops_off, n, score_only)
        assert np.array_equal(got[0], exp[0]), f"scores differ on call {call}"
        assert np.array_equal(got[1], exp[1]), f"status differs on call {call}"
        if not score_only:
            bad = [i for i in range(n) if got[2][i] != exp[2][i]]
            assert not bad, f"CIGARs differ on call {call}: pairs {bad[:5]}"
    al.close()


def test_noalloc_backtrace_limit_reports_oom():
    """A pair whose back-trace needs more than the 512 KiB per warp reports
    WF_STATUS_OOM with no CIGAR; the other pairs of the batch are unaffected."""
    torch = pytest.importorskip("torch")
    import helpers
    import wfa2gpu as W
    W.build()
    g = W.generate(1, 40, first=99)
    pats = [g.pattern(i) for i in range(g.n)]
    txts = [g.text(i) for i in range(g.n)]
    rng = np.random.default_rng(7)
    big = 20  # two unrelated 2 kbp sequences: millions of cells
    acgt = np.frombuffer(b"ACGT", np.uint8)
    pats.insert(big, rng.choice(acgt, 2000).tobytes())
    txts.insert(big, rng.choice(acgt, 2000).tobytes())
    seqs, po, pl, to, tl = helpers.pack(pats, txts)
    p = W.Pairs(seqs, po, pl, to, tl)
    n = len(pats)
    d, ops_off = _device_batch(torch, W, p)
    al = W.Aligner(W.Config())
    ref = _outputs(torch, n, int(ops_off[-1]))
    assert _run(al, False, n, d, ref, int(max(pl.max(), tl.max())), False, 0) == 0
    out = _outputs(torch, n, int(ops_off[-1]))
    assert _run(al, True, n, d, out, int(max(pl.max(), tl.max())), False, 0) == 0
    torch.cuda.synchronize()
    exp = _host(ref, ops_off, n, False)
    got = _host(out, ops_off, n, False)
    assert exp[1][big] == 0
    assert got[1][big] == W.WF_STATUS_OOM and len(got[2][big]) == 0
    others = [i for i in range(n) if i != big]
    assert np.array_equal(got[0][others], exp[0][others])
    assert np.array_equal(got[1][others], exp[1][others])
    assert all(got[2][i] == exp[2][i] for i in others)
    al.close()


def test_noalloc_rejects_sequences_beyond_its_limit():
    torch = pytest.importorskip("torch")
    import wfa2gpu as W
    W.build()
    p = W.generate(5, 4, param=3000, param2=20)
    d, ops_off = _device_batch(torch, W, p)
    o = _outputs(torch, p.n, int(ops_off[-1]))
    al = W.Aligner(W.Config())
    assert _run(al, True, p.n, d, o, p.max_len, False, 0) == WF2G_ERR_ARGS
    al.close()

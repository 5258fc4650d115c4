"""BiWFA (ultralow memory mode) on the GPU against the CPU checker: the
breakpoint-search kernel, the level-by-level recursion and the base cases
with begin/end components, through the C ABI.  Integer work: scores, statuses
and CIGARs must be identical; every CIGAR is replayed and rescored."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

UT = helpers.utest_expected()
MEM_ULTRALOW = 3


def _cfg(W, spec, score_only, max_steps=0):
    m, match, x, o1, e1, o2, e2 = spec
    return W.Config(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                    gap_opening2=o2, gap_extension2=e2, score_only=score_only,
                    memory_mode=MEM_ULTRALOW, max_steps=max_steps)


def _pen(O, spec):
    m, match, x, o1, e1, o2, e2 = spec
    return O.Penalties(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                       gap_opening2=o2, gap_extension2=e2)


def _gpu(W, cfg, seqs, p_off, p_len, t_off, t_len):
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(seqs, p_off, p_len, t_off, t_len)
    launches = al.launches
    al.close()
    assert rc == 0
    assert launches >= 2  # packing + at least one breakpoint search
    cig = None
    if not cfg.score_only:
        cig = [ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode() for i in range(len(p_len))]
    return scores, status, cig


def _compare(O, W, spec, batch, score_only, max_steps=0):
    seqs, p_off, p_len, t_off, t_len = batch
    scores, status, cig = _gpu(W, _cfg(W, spec, score_only, max_steps), *batch)
    b = O.PairBatch(seqs, p_off, p_len, t_off, t_len)
    r = O.align(b, _pen(O, spec), memory_mode=MEM_ULTRALOW, score_only=score_only,
                max_steps=max_steps)
    bad = [i for i in range(len(p_len)) if scores[i] != r.score[i] or status[i] != r.status[i]]
    assert not bad, [(i, int(scores[i]), int(r.score[i]), int(status[i]), int(r.status[i]))
                     for i in bad[:5]]
    if cig is not None:
        pen = _pen(O, spec)
        for i in range(len(p_len)):
            assert cig[i] == r.cigar(i), i
            if status[i] == 0:
                assert O.check_cigar(cig[i], b.pattern(i), b.text(i)), i
                # an empty pattern or text is a trivial top-level case: the
                # reference leaves cigar->score at its cleared value INT32_MIN
                # (wavefront/wavefront_bialign.c:1155-1161)
                if scores[i] != np.iinfo(np.int32).min:
                    assert O.rescore(cig[i], pen) == int(scores[i]), i


@pytest.mark.parametrize("spec_name", ["affine", "affine2p", "affine.p3", "affine.p1"])
@pytest.mark.parametrize("score_only", [False, True])
def test_bialign_matches_oracle(gpu_available, wfa, oracle_mod, spec_name, score_only):
    W, O = wfa, oracle_mod
    p = W.generate(5, 24, param=2500, param2=250, first=777)
    _compare(O, W, UT["penalty_sets"][spec_name], (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len),
             score_only)


@pytest.mark.parametrize("max_steps", [40, 400, 900])
def test_bialign_max_steps(gpu_available, wfa, oracle_mod, max_steps):
    W, O = wfa, oracle_mod
    p = W.generate(5, 24, param=1500, param2=150, first=99)
    batch = (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    for so in (False, True):
        _compare(O, W, UT["penalty_sets"]["affine"], batch, so, max_steps)


def test_bialign_edge_cases(gpu_available, wfa, oracle_mod):
    """Empty sequences, identical long sequences (end reached at score 0),
    short pairs (base case at once), non-ACGT bytes (byte comparisons), a
    long insertion that splits inside a gap component."""
    W, O = wfa, oracle_mod
    rng = np.random.default_rng(5)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    rand = lambda n: acgt[rng.integers(0, 4, n)].tobytes()
    long_a = rand(3000)
    with_n = bytearray(rand(2500))
    for j in range(0, 2500, 97):
        with_n[j] = ord("N")
    with_n = bytes(with_n)
    with_n_t = bytearray(with_n)
    for j in range(5, 2500, 41):
        with_n_t[j] = ord("ACGT"[j % 4])
    gap_t = long_a[:1500] + rand(300) + long_a[1500:]
    pats = [b"", b"A", b"", long_a, b"ACGTACGT", with_n, long_a, rand(700), long_a[:2000]]
    txts = [b"", b"", b"ACG", long_a, b"ACGAACGT", bytes(with_n_t), gap_t, rand(650), b""]
    batch = helpers.pack(pats, txts)
    for spec in ("affine", "affine2p"):
        for so in (False, True):
            _compare(O, W, UT["penalty_sets"][spec], batch, so)


def test_bialign_per_pair_and_device_entry_points(gpu_available, wfa, oracle_mod):
    """wavefront_align() and wavefront_align_batch_device() in ultralow mode
    give the batch results."""
    torch = pytest.importorskip("torch")
    W, O = wfa, oracle_mod
    p = W.generate(5, 6, param=2000, param2=200, first=3)
    batch = (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    cfg = _cfg(W, UT["penalty_sets"]["affine"], False)
    scores, status, cig = _gpu(W, cfg, *batch)
    al = W.Aligner(cfg)
    for i in range(p.n):
        st, sc, ops = al.align(p.pattern(i), p.text(i))
        assert (st, sc, ops) == (int(status[i]), int(scores[i]), cig[i]), i
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    cap = p.p_len.astype(np.int64) + p.t_len.astype(np.int64)
    ops_off = np.zeros(p.n + 1, np.int64)
    np.cumsum(cap, out=ops_off[1:])
    d_seqs, d_po, d_pl, d_to, d_tl = map(T, batch)
    d_oo = T(ops_off)
    d_sc = torch.zeros(p.n, dtype=torch.int32, device=dev)
    d_st = torch.zeros(p.n, dtype=torch.int32, device=dev)
    d_ol = torch.zeros(p.n, dtype=torch.int32, device=dev)
    d_ops = torch.zeros(int(ops_off[-1]) + 16, dtype=torch.uint8, device=dev)
    rc = al.align_batch_device(p.n, d_seqs.data_ptr(), d_po.data_ptr(), d_pl.data_ptr(),
                               d_to.data_ptr(), d_tl.data_ptr(), p.max_len, d_sc.data_ptr(),
                               d_st.data_ptr(), d_ops.data_ptr(), d_oo.data_ptr(),
                               d_ol.data_ptr(), 0)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_sc.cpu().numpy(), scores)
    assert np.array_equal(d_st.cpu().numpy(), status)
    ops_h = d_ops.cpu().numpy()
    ol = d_ol.cpu().numpy()
    for i in range(p.n):
        assert ops_h[ops_off[i]:ops_off[i] + ol[i]].tobytes().decode() == cig[i], i
    al.close()


def test_biwfa_cigar_end_position(gpu_available, wfa, oracle_mod):
    """wavefront_align() in ultralow mode leaves cigar->end_v/end_h where the
    reference does: the sequence lengths after a score-only search or a
    top-level split, (-1,-1) when the whole pair went to the base case
    (wavefront/wavefront_bialign.c:159-194, :1214-1220, :1248-1257)."""
    W, O = wfa, oracle_mod
    for wl, n, pa, pb in [(0, 40, 0, 0), (1, 30, 0, 0)]:
        p = W.generate(wl, n, param=pa, param2=pb)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        for metric in (W.GAP_AFFINE, W.GAP_AFFINE_2P):
            for so in (False, True):
                pen = O.Penalties(metric)
                r = O.align(b, pen, memory_mode=O.MEM_ULTRALOW, score_only=so)
                al = W.Aligner(W.Config(metric=metric, memory_mode=W.MEM_ULTRALOW, score_only=so))
                for i in range(b.n):
                    st, score, _ = al.align(b.pattern(i), b.text(i))
                    cg = al._h.contents.cigar.contents
                    assert (st, score, cg.end_v, cg.end_h) == (
                        int(r.status[i]), int(r.score[i]), int(r.end[i][0]), int(r.end[i][1])), \
                        (wl, metric, so, i)
                al.close()

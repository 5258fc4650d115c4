"""Heuristic cut-offs other than wf-adaptive on the GPU, through the C ABI.

Strategies (wavefront/wavefront_heuristic.c:229-563): wfmash, x-drop, z-drop,
banded static and banded adaptive, alone and combined (one of wf-adaptive /
wfmash, one of x-drop / z-drop, one of the bands, sharing one wait counter).

Integer work: scores, statuses, CIGARs and end positions must equal the
reference's own outputs (tests/golden/heuristics_expected.json) and the CPU
checker's on further cases, for every pair except one documented class: a
back-trace that takes a source from a wavefront a cut emptied, which the
reference's compute step read as NULL but its back-trace reads cell by cell
(wavefront/wavefront_backtrace.c:63-100).  Where that source lies ahead of
the cell, the reference takes back CIGAR operations it already wrote; the GPU
records each cell's own source instead.  The CPU checker flags those pairs
(FLAG_STALE_SOURCE); they are counted, not compared.

Configurations the GPU does not compute yet (z-drop with a full alignment,
z-drop with gap-affine-2p) must be refused: WF2G_ERR_CONFIG for a batch."""
import pytest

import helpers

pytestmark = pytest.mark.gpu

UT = helpers.utest_expected()
HX = helpers.heuristics_expected()


def _spec(name):
    m, match, x, o1, e1, o2, e2 = UT["penalty_sets"][name]
    return dict(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                gap_opening2=o2, gap_extension2=e2)


def _served(metric, score_only, strategy, memory_mode=0):
    """The GPU's refusals (make_cfg in wfa2-lib_gb300/csrc/wfa_aligner.c)."""
    return not (memory_mode == 3 and strategy & 0x20)  # BiWFA: no z-drop


def _gpu(W, cfg, b):
    """Status, score, CIGAR and end position per pair (BiWFA: no end position,
    which the ends call does not serve there: -1, -1)."""
    al = W.Aligner(cfg)
    if cfg.memory_mode == 3:
        rc, scores, status, ops, ops_len, ops_off = al.align_batch(
            b.seqs, b.p_off, b.p_len, b.t_off, b.t_len)
        end = [(-1, -1)] * b.n
    else:
        rc, scores, status, ops, ops_len, ops_off, end = al.align_batch_ends(
            b.seqs, b.p_off, b.p_len, b.t_off, b.t_len)
    al.close()
    if not _served(cfg.metric, cfg.score_only, cfg.heuristic["strategy"], cfg.memory_mode):
        assert rc == -2  # WF2G_ERR_CONFIG: refused, no answer
        return None
    assert rc == 0
    out = []
    for i in range(b.n):
        cig = ("" if ops is None or cfg.score_only
               else ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode())
        out.append((int(status[i]), int(scores[i]), cig, int(end[i][0]), int(end[i][1])))
    return out


def _oracle_flags(O, pen_spec, b, score_only, form, hspec, max_steps=0):
    pen = O.Penalties(**{"metric": pen_spec["metric"], "match": pen_spec["match"],
                         "mismatch": pen_spec["mismatch"],
                         "gap_opening1": pen_spec["gap_opening1"],
                         "gap_extension1": pen_spec["gap_extension1"],
                         "gap_opening2": pen_spec["gap_opening2"],
                         "gap_extension2": pen_spec["gap_extension2"]})
    return O.align(b, pen, score_only=score_only, form=form, heuristic=O.Heuristic(**hspec),
                   max_steps=max_steps)


@pytest.mark.parametrize("name", sorted(HX.keys()))
def test_heuristics_match_reference_fixtures(gpu_available, wfa, oracle_mod, name):
    W, O = wfa, oracle_mod
    fx = HX[name]
    spec = _spec(fx["penalties"])
    b = helpers.heuristic_pairs(O, W, fx)
    ref = _oracle_flags(O, spec, b, fx["score_only"], fx["form"], fx["heuristic"],
                        max_steps=fx.get("max_steps", 0))
    got = _gpu(W, W.Config(**spec, score_only=fx["score_only"], form=fx["form"],
                           heuristic=fx["heuristic"], memory_mode=fx.get("memory_mode", 0),
                           max_steps=fx.get("max_steps", 0)), b)
    if got is None:
        return
    compared = 0
    for i, (score, status, c, ev, eh) in enumerate(fx["rows"]):
        if ref.flags[i] & O.FLAG_STALE_SOURCE:
            continue
        st, sc, cig, gv, gh = got[i]
        if fx.get("memory_mode", 0) == 3:
            assert (st, sc, helpers.crc(cig)) == (status, score, c), (name, i)
        else:
            assert (st, sc, helpers.crc(cig), gv, gh) == (status, score, c, ev, eh), (name, i)
        compared += 1
    assert compared >= len(fx["rows"]) // 2, (name, compared)


CASES = [
    # (workload, n, param, param2)
    (1, 120, 0, 0),          # 0.5-1.5 kbp, warp per pair
    (6, 120, 0, 0),          # random tails: the drops fire
    (5, 16, 6000, 300),      # 6 kbp: the CTA-per-pair passes
]
H = {
    "bstatic": dict(strategy=0x01, min_k=-40, max_k=40),
    "badapt": dict(strategy=0x02, min_k=-25, max_k=25, steps_between_cutoffs=2),
    "wfmash": dict(strategy=0x40, min_wavefront_length=10, max_distance_threshold=50,
                   steps_between_cutoffs=1),
    "xdrop": dict(strategy=0x10, xdrop=80, steps_between_cutoffs=1),
    "zdrop": dict(strategy=0x20, zdrop=80, steps_between_cutoffs=1),
    "wfa_xdrop_band": dict(strategy=0x04 | 0x10 | 0x01, min_wavefront_length=10,
                           max_distance_threshold=50, xdrop=100, min_k=-60, max_k=60,
                           steps_between_cutoffs=1),
}


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("hname", sorted(H.keys()))
@pytest.mark.parametrize("spec_name,score_only", [("affine.p4", False), ("affine2p", False),
                                                  ("affine.p4", True)])
def test_heuristics_match_oracle(gpu_available, wfa, oracle_mod, case, hname, spec_name,
                                 score_only):
    W, O = wfa, oracle_mod
    wl, n, param, param2 = case
    spec = _spec(spec_name)
    p = W.generate(wl, n, param=param, param2=param2)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    ref = _oracle_flags(O, spec, b, score_only, None, H[hname])
    got = _gpu(W, W.Config(**spec, score_only=score_only, heuristic=H[hname]), b)
    if got is None:
        return
    compared = 0
    for i in range(b.n):
        if ref.flags[i] & (O.FLAG_STALE_SOURCE | O.FLAG_OVER_BOUND):
            continue
        want = (int(ref.status[i]), int(ref.score[i]), ref.cigar(i), int(ref.end[i][0]),
                int(ref.end[i][1]))
        assert got[i] == want, (hname, spec_name, case, i)
        compared += 1
    assert compared >= b.n // 2, (hname, compared)


def test_heuristic_rejections(gpu_available, wfa):
    """Drops with edit/indel (the reference exits, wavefront/wavefront_align.c:
    83-89), BiWFA with z-drop, and serving with a heuristic other than
    wf-adaptive are refused loudly."""
    W = wfa
    p = W.generate(1, 4, first=3)
    for cfg in [W.Config(metric=W.EDIT, heuristic=dict(strategy=0x10, xdrop=20)),
                W.Config(metric=W.INDEL, heuristic=dict(strategy=0x20, zdrop=20)),
                W.Config(memory_mode=W.MEM_ULTRALOW, heuristic=dict(strategy=0x20, zdrop=50))]:
        al = W.Aligner(cfg)
        st, _, _ = al.align(bytes(p.seqs[p.p_off[0]:p.p_off[0] + p.p_len[0]]),
                            bytes(p.seqs[p.t_off[0]:p.t_off[0] + p.t_len[0]]))
        al.close()
        assert st == W.WF_STATUS_UNATTAINABLE
    with pytest.raises(RuntimeError):
        W.Server(W.Config(heuristic=dict(strategy=0x10, xdrop=20)))


@pytest.mark.parametrize("hname", sorted(k for k in H if k != "zdrop"))
@pytest.mark.parametrize("spec_name,score_only", [("affine", False), ("affine2p", False),
                                                  ("affine.p4", True), ("linear", False)])
@pytest.mark.parametrize("wl", [1, 6])
def test_biwfa_heuristics_match_oracle(gpu_available, wfa, oracle_mod, hname, spec_name,
                                       score_only, wl):
    """BiWFA (ultralow memory): the forward and reverse breakpoint searches
    inherit the heuristic (wavefront/wavefront_bialigner.c:48-56), each
    direction with its own wait counter and x-drop best, cleared at every
    search, and each step's range widened by its null inputs as the
    reference's is; the base cases take none.  Scores, statuses and CIGARs
    equal the checker's (0.5-1.5 kbp pairs, and random-tail pairs where the
    cuts end searches)."""
    W, O = wfa, oracle_mod
    spec = _spec(spec_name)
    p = W.generate(wl, 40, first=5)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    pen = O.Penalties(**spec)
    ref = O.align(b, pen, memory_mode=O.MEM_ULTRALOW, score_only=score_only,
                  heuristic=O.Heuristic(**H[hname]))
    got = _gpu(W, W.Config(**spec, memory_mode=W.MEM_ULTRALOW, score_only=score_only,
                           heuristic=H[hname]), b)
    if got is None:  # refused (asserted in _gpu)
        return
    compared = 0
    for i in range(b.n):
        if ref.flags[i] & (O.FLAG_STALE_SOURCE | O.FLAG_OVER_BOUND):
            continue
        assert got[i][:3] == (int(ref.status[i]), int(ref.score[i]), ref.cigar(i)), \
            (hname, spec_name, wl, i)
        compared += 1
    assert compared >= b.n // 2


@pytest.mark.parametrize("case", CASES[:2])
@pytest.mark.parametrize("spec_name", ["linear", "linear.m1", "affine", "affine2p"])
def test_zdrop_full_alignment_matches_oracle(gpu_available, wfa, oracle_mod, case, spec_name):
    """z-drop with a full alignment on gap-linear, gap-affine and
    gap-affine-2p (match 0 and < 0): the walk from the best cell (its first step from the sources of the
    current score, wavefront/wavefront_backtrace.c:62-219), the gaps to both
    ends and the maximal-score trim, against the checker."""
    W, O = wfa, oracle_mod
    wl, n, param, param2 = case
    spec = _spec(spec_name)
    p = W.generate(wl, n, param=param, param2=param2)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    hs = dict(strategy=0x20, zdrop=60, steps_between_cutoffs=1)
    ref = _oracle_flags(O, spec, b, False, None, hs)
    got = _gpu(W, W.Config(**spec, heuristic=hs), b)
    compared = 0
    for i in range(b.n):
        if ref.flags[i] & (O.FLAG_STALE_SOURCE | O.FLAG_OVER_BOUND):
            continue
        want = (int(ref.status[i]), int(ref.score[i]), ref.cigar(i), int(ref.end[i][0]),
                int(ref.end[i][1]))
        assert got[i] == want, (spec_name, case, i)
        compared += 1
    assert compared >= b.n // 2, (spec_name, compared)


@pytest.mark.parametrize("params", [(10, 50, 1), (20, 30, 2), (1, 0, 3), (5, 10, 1)])
@pytest.mark.parametrize("score_only", [False, True])
def test_wfadaptive_fast_pass_matches_oracle(gpu_available, wfa, oracle_mod, params, score_only):
    """wf-adaptive alone on the default penalties runs in the two-diagonal
    fast kernel (cut-off after the termination test, limits shrunk, the cut
    cells kept readable in the rows' windows): every pair the checker does
    not flag as reading a cut-emptied source equals the checker, on a batch
    of 0.5-1.5 kbp pairs and on random-tail pairs where the cuts fire."""
    W, O = wfa, oracle_mod
    for wl, n in [(1, 600), (6, 120)]:
        p = W.generate(wl, n, first=77)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        al = W.Aligner(W.Config(score_only=score_only, wfadaptive=params))
        rc, scores, status, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len,
                                                                   p.t_off, p.t_len)
        al.close()
        assert rc == 0
        r = O.align(b, O.Penalties(), score_only=score_only, wfadaptive=params)
        compared = 0
        for i in range(n):
            if r.flags[i] & O.FLAG_STALE_SOURCE:
                continue
            got = (int(status[i]), int(scores[i]))
            assert got == (int(r.status[i]), int(r.score[i])), (params, wl, i)
            if not score_only:
                assert ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode() == r.cigar(i), \
                    (params, wl, i)
            compared += 1
        assert compared >= n // 2


@pytest.mark.parametrize("params", [None, (20, 30, 2), (1, 0, 3)])
@pytest.mark.parametrize("score_only", [False, True])
def test_wider_passes_match_oracle(gpu_available, wfa, oracle_mod, monkeypatch, params,
                                   score_only):
    """With the first fast pass narrowed to diagonals [-32, 32]
    (WF2G_FAST_REACH), it sends most pairs to the wider passes: the second
    and third passes then align most of the batch, with and without the
    wf-adaptive cut-off, and equal the checker."""
    W, O = wfa, oracle_mod
    monkeypatch.setenv("WF2G_FAST_REACH", "32")
    n = 600
    p = W.generate(1, n, first=77)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    al = W.Aligner(W.Config(score_only=score_only, wfadaptive=params))
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len,
                                                               p.t_off, p.t_len)
    al.close()
    assert rc == 0
    r = O.align(b, O.Penalties(), score_only=score_only, wfadaptive=params)
    compared = 0
    for i in range(n):
        if r.flags[i] & O.FLAG_STALE_SOURCE:
            continue
        assert (int(status[i]), int(scores[i])) == (int(r.status[i]), int(r.score[i])), (params, i)
        if not score_only:
            assert ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode() == r.cigar(i), \
                (params, i)
        compared += 1
    assert compared >= n // 2

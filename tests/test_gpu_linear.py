"""The single-component metrics -- indel, edit and gap-linear -- on the GPU,
through the C ABI, against the CPU checker.

The reference computes them with one M wavefront per score
(wavefront/wavefront_compute_edit.c, wavefront/wavefront_compute_linear.c) and
a one-state back-trace (wavefront/wavefront_backtrace.c:223-319).  The GPU
runs them on the gap-affine recurrence with no gap-extension wavefronts, plus
the edit driver's particulars:
- indel has no mismatch;
- the score is the distance itself;
- end-to-end edit prunes wavefronts of 1000 or more diagonals;
- edit and indel are not trimmed in the extension form.

Golden coverage (the reference test-suite's edit/indel files, BiWFA
included, and reference outputs for gap-linear and the pruning cases) is in
test_gpu_parity.py.
Integer work: everything must be identical."""
import pytest

import helpers

pytestmark = pytest.mark.gpu

PENS = {
    "indel": dict(metric=0),
    "edit": dict(metric=1),
    "linear": dict(metric=2, match=0, mismatch=4, gap_opening1=2),
    "linear.m1": dict(metric=2, match=-1, mismatch=3, gap_opening1=2),
}
CASES = [
    (1, 200, 0, 0),        # 0.5-1.5 kbp
    (5, 12, 6000, 200),    # 6 kbp at 20 %: the CTA-per-pair passes, wide wavefronts
    (6, 8, 3000, 200),     # very different lengths: edit pruning
]


def _gpu(W, cfg, p, ends=False):
    al = W.Aligner(cfg)
    if ends:
        rc, scores, status, ops, ops_len, ops_off, end = al.align_batch_ends(
            p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    else:
        rc, scores, status, ops, ops_len, ops_off = al.align_batch(
            p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        end = None
    al.close()
    assert rc == 0
    out = []
    for i in range(p.n):
        cig = "" if cfg.score_only else ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode()
        e = (int(end[i][0]), int(end[i][1])) if ends else None
        out.append((int(status[i]), int(scores[i]), cig, e))
    return out


def _oracle(O, pen, p, **kw):
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, O.Penalties(**pen), **kw)
    return r


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("name", sorted(PENS))
@pytest.mark.parametrize("score_only", [False, True])
@pytest.mark.parametrize("heur", [None, (10, 50, 1)])
def test_linear_metrics_match_oracle(gpu_available, wfa, oracle_mod, case, name, score_only,
                                     heur):
    W, O = wfa, oracle_mod
    wl, n, param, param2 = case
    p = W.generate(wl, n, first=4321, param=param, param2=param2)
    pen = PENS[name]
    got = _gpu(W, W.Config(**pen, score_only=score_only, wfadaptive=heur), p)
    r = _oracle(O, pen, p, score_only=score_only, wfadaptive=heur)
    for i in range(n):
        assert got[i][:3] == (int(r.status[i]), int(r.score[i]), r.cigar(i)), (name, i)


@pytest.mark.parametrize("name", sorted(PENS))
@pytest.mark.parametrize("form", [(0, 30, 0, 30), (20, 20, 20, 20), "extension"])
def test_linear_metrics_endsfree(gpu_available, wfa, oracle_mod, name, form):
    W, O = wfa, oracle_mod
    pen = PENS[name]
    if form != "extension" and (form[0] or form[2]) and (pen["metric"] <= 1 or pen.get("match")):
        pytest.skip("begin-free lengths: edit/indel and match < 0 are not served")
    p = W.generate(1, 150, first=99)
    got = _gpu(W, W.Config(**pen, form=form), p, ends=True)
    r = _oracle(O, pen, p, form=form)
    for i in range(p.n):
        want = (int(r.status[i]), int(r.score[i]), r.cigar(i),
                (int(r.end[i][0]), int(r.end[i][1])))
        assert got[i] == want, (name, form, i)


@pytest.mark.parametrize("name", ["indel", "edit"])
@pytest.mark.parametrize("form", [(20, 20, 20, 20), (0, 0, 60, 5), (45, 0, 0, 0)])
@pytest.mark.parametrize("case", [(1, 150, 0, 0), (5, 40, 400, 300), (6, 8, 3000, 200)])
def test_edit_indel_begin_free_score_only(gpu_available, wfa, oracle_mod, name, form, case):
    """Edit and indel with begin-free lengths, score only: M[0] spans
    [-pattern_begin_free, text_begin_free] and the edit driver reads it by its
    limits (wavefront/wavefront_aligner.c:250-305,
    wavefront/wavefront_compute_edit.c:321-374); score, status and end
    position equal the checker's."""
    W, O = wfa, oracle_mod
    wl, n, param, param2 = case
    pen = PENS[name]
    p = W.generate(wl, n, first=57, param=param, param2=param2)
    got = _gpu(W, W.Config(**pen, form=form, score_only=True), p, ends=True)
    r = _oracle(O, pen, p, form=form, score_only=True)
    for i in range(p.n):
        want = (int(r.status[i]), int(r.score[i]), "", (int(r.end[i][0]), int(r.end[i][1])))
        assert got[i] == want, (name, form, case, i)


def test_linear_metrics_dropin(gpu_available, wfa, oracle_mod):
    """wavefront_align() per pair with edit and gap-linear attributes."""
    W, O = wfa, oracle_mod
    p = W.generate(0, 40, first=7)
    for name in ("edit", "linear"):
        pen = PENS[name]
        al = W.Aligner(W.Config(**pen))
        r = _oracle(O, pen, p)
        for i in range(p.n):
            st, score, ops = al.align(p.pattern(i), p.text(i))
            assert (st, score, ops) == (int(r.status[i]), int(r.score[i]), r.cigar(i)), (name, i)
        al.close()


@pytest.mark.parametrize("name", sorted(PENS))
@pytest.mark.parametrize("case", [(1, 100, 0, 0), (5, 12, 3000, 200), (6, 6, 3000, 150)])
@pytest.mark.parametrize("score_only", [False, True])
def test_linear_metrics_biwfa(gpu_available, wfa, oracle_mod, name, case, score_only):
    """BiWFA (ultralow memory) for the single-component metrics: only M-to-M
    breakpoints, no gap-open adjustment, edit pruning inside the breakpoint
    searches and base cases (wavefront/wavefront_bialign.c:83-150, :878-973)."""
    W, O = wfa, oracle_mod
    wl, n, param, param2 = case
    p = W.generate(wl, n, first=31, param=param, param2=param2)
    pen = PENS[name]
    got = _gpu(W, W.Config(**pen, memory_mode=W.MEM_ULTRALOW, score_only=score_only), p)
    r = _oracle(O, pen, p, memory_mode=O.MEM_ULTRALOW, score_only=score_only)
    for i in range(n):
        assert got[i][:3] == (int(r.status[i]), int(r.score[i]), r.cigar(i)), (name, i)


def test_linear_metrics_rejections(gpu_available, wfa):
    """Edit/indel begin-free lengths with a full alignment are not served
    (score only is); serving takes the gap-affine metrics only."""
    W = wfa
    p = W.generate(1, 4, first=3)
    for cfg in [W.Config(metric=0, form=(5, 5, 5, 5))]:
        al = W.Aligner(cfg)
        rc = al.align_batch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)[0]
        al.close()
        assert rc == -2  # WF2G_ERR_CONFIG
    with pytest.raises(RuntimeError):
        W.Server(W.Config(metric=1))

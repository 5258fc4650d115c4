"""Ends-free and extension alignment forms on the GPU, through the C ABI.

Semantics (wavefront/wavefront_attributes.h:55-69):
- ends-free with match 0: the score-0 wavefront spans the begin-free
  diagonals (wavefront/wavefront_aligner.c:250-305);
- termination: the first diagonal, in extension order, that reaches the end
  of one sequence with the other's rest within its end-free length
  (wavefront/wavefront_termination.c:115-162);
- the CIGAR spans both sequences, with the free ends as I/D runs
  (wavefront/wavefront_backtrace.c:346-356, :506-516);
- extension: the ends-free presets, then maximal-score trimming
  (wavefront/wavefront_align.c:57-63, alignment/cigar_utils.c:112-318).

Integer work: scores, statuses, CIGARs and end positions must be identical to
the reference's own outputs (tests/golden/endsfree_expected.json, from the
reference's portable build) and to the CPU checker on further cases."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

UT = helpers.utest_expected()
EF = helpers.endsfree_expected()


def _spec(name):
    m, match, x, o1, e1, o2, e2 = UT["penalty_sets"][name]
    return dict(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                gap_opening2=o2, gap_extension2=e2)


def _gpu(W, cfg, p):
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off, end = al.align_batch_ends(
        p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    al.close()
    assert rc == 0
    out = []
    for i in range(p.n):
        cig = "" if ops is None else ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode()
        out.append((int(status[i]), int(scores[i]), cig, int(end[i][0]), int(end[i][1])))
    return out


@pytest.mark.parametrize("name", sorted(EF.keys()))
def test_endsfree_matches_reference_fixtures(gpu_available, wfa, name):
    W = wfa
    fx = EF[name]
    p = W.generate(fx["workload"], fx["n"], param=fx["param"], param2=fx["param2"])
    cfg = W.Config(**_spec(fx["penalties"]), score_only=fx["score_only"], form=fx["form"],
                   wfadaptive=fx["wfadaptive"])
    got = _gpu(W, cfg, p)
    for i, (score, status, c, ev, eh) in enumerate(fx["rows"]):
        st, sc, cig, gv, gh = got[i]
        assert (st, sc, helpers.crc(cig), gv, gh) == (status, score, c, ev, eh), (name, i)


CASES = [
    # (workload, n, param, param2)
    (1, 200, 0, 0),           # 0.5-1.5 kbp, warp per pair
    (5, 24, 6000, 120),       # 6 kbp: the CTA-per-pair passes
    (5, 40, 400, 300),        # short, 30 % divergence
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("spec_name", ["affine", "affine2p", "affine.p3"])
@pytest.mark.parametrize("form", [(7, 7, 7, 7), (0, 60, 0, 60), (30, 0, 0, 30), "extension"])
@pytest.mark.parametrize("score_only", [False, True])
def test_endsfree_matches_oracle(gpu_available, wfa, oracle_mod, case, spec_name, form,
                                 score_only):
    W, O = wfa, oracle_mod
    spec = _spec(spec_name)
    wl, n, param, param2 = case
    p = W.generate(wl, n, first=1234, param=param, param2=param2)
    got = _gpu(W, W.Config(**spec, score_only=score_only, form=form), p)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, O.Penalties(**spec), score_only=score_only, form=form)
    for i in range(n):
        want = (int(r.status[i]), int(r.score[i]), r.cigar(i), int(r.end[i][0]),
                int(r.end[i][1]))
        assert got[i] == want, (spec_name, form, i)


def test_endsfree_with_wfadaptive_matches_oracle(gpu_available, wfa, oracle_mod):
    W, O = wfa, oracle_mod
    p = W.generate(5, 40, first=77, param=2000, param2=100)
    for form in [(10, 10, 10, 10), "extension"]:
        got = _gpu(W, W.Config(form=form, wfadaptive=(10, 50, 1)), p)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        r = O.align(b, O.Penalties(), form=form, wfadaptive=(10, 50, 1))
        for i in range(p.n):
            assert got[i] == (int(r.status[i]), int(r.score[i]), r.cigar(i),
                              int(r.end[i][0]), int(r.end[i][1])), (form, i)


def test_endsfree_dropin_cigar_fields(gpu_available, wfa, oracle_mod):
    """wavefront_align() with free ends: cigar->end_v/end_h and align_status.score
    as the reference fills them (wavefront/wavefront_unialign.c:147-237)."""
    W, O = wfa, oracle_mod
    p = W.generate(1, 30, first=500)
    for form in [(20, 20, 20, 20), "extension"]:
        cfg = W.Config(form=form)
        attr = cfg.attributes()
        wf = W.lib().wavefront_aligner_new(attr)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        r = O.align(b, O.Penalties(), form=form)
        for i in range(p.n):
            P, T = p.pattern(i), p.text(i)
            st = W.lib().wavefront_align(wf, P, len(P), T, len(T))
            cg = wf.contents.cigar.contents
            ops = b""
            if cg.end_offset > cg.begin_offset:
                ops = bytes(cg.operations[cg.begin_offset:cg.end_offset])
            assert (st, cg.score, ops.decode(), cg.end_v, cg.end_h) == (
                int(r.status[i]), int(r.score[i]), r.cigar(i), int(r.end[i][0]),
                int(r.end[i][1])), (form, i)
        W.lib().wavefront_aligner_delete(wf)


def test_endsfree_rejections(gpu_available, wfa):
    """Forms the GPU path does not serve fail loudly: BiWFA with free ends (the
    reference exits, wavefront/wavefront_align.c:67-82), edit/indel with
    begin-free lengths and a full alignment (the reference's back-trace reads
    the begin-free diagonals as sourceless; their score-only form is served),
    and serving with free ends (its BiWFA fallback)."""
    W = wfa
    p = W.generate(1, 4, first=3)
    for cfg in [W.Config(form=(5, 5, 5, 5), memory_mode=W.MEM_ULTRALOW),
                W.Config(metric=W.EDIT, form=(5, 0, 0, 0)),
                W.Config(metric=W.INDEL, form=(0, 0, 5, 0))]:
        al = W.Aligner(cfg)
        rc = al.align_batch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)[0]
        al.close()
        assert rc == -2  # WF2G_ERR_CONFIG
    with pytest.raises(RuntimeError):
        W.Server(W.Config(form=(5, 5, 5, 5)))

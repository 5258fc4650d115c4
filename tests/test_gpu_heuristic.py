"""The wf-adaptive heuristic (the reference's default attributes,
wavefront/wavefront_attributes.c:71-76) on the GPU against the CPU checker.

The heuristic cuts each extended M wavefront after every few steps.  Cut-off
offsets stay readable by later steps and by the back-trace.  Modes covered:
high, score-only and BiWFA.  Integer work, so scores and statuses must be
identical.  CIGARs must also be identical wherever the checker's CIGAR is a
valid alignment of the pair.

Rare case: under this heuristic the reference's back-trace can emit a CIGAR
that does not align the pair.  It reads cut-off offsets of a gap wavefront
whose limits the cut-off emptied (wavefront/wavefront_backtrace.c:63-219).
Where the checker's CIGAR is invalid for that reason, the GPU must return the
same score and status and a valid CIGAR of that score."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

UT = helpers.utest_expected()


def _spec(name):
    m, match, x, o1, e1, o2, e2 = UT["penalty_sets"][name]
    return dict(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                gap_opening2=o2, gap_extension2=e2)


@pytest.mark.parametrize("workload,n,param,param2", [(1, 300, 0, 0), (2, 12, 0, 0),
                                                      (5, 40, 3000, 300)])
@pytest.mark.parametrize("spec_name", ["affine", "affine2p", "affine.p3"])
@pytest.mark.parametrize("heur", [(10, 50, 1), (10, 50, 10), (4, 10, 3)])
@pytest.mark.parametrize("mode,score_only", [(0, False), (0, True), (3, False)])
def test_wfadaptive_matches_oracle(gpu_available, wfa, oracle_mod, workload, n, param, param2,
                                   spec_name, heur, mode, score_only):
    W, O = wfa, oracle_mod
    p = W.generate(workload, n, first=321, param=param, param2=param2)
    cfg = W.Config(**_spec(spec_name), score_only=score_only, memory_mode=mode, wfadaptive=heur)
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len,
                                                              p.t_off, p.t_len)
    al.close()
    assert rc == 0
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    pen = O.Penalties(**_spec(spec_name))
    r = O.align(b, pen, memory_mode=mode, score_only=score_only, wfadaptive=heur)
    assert np.array_equal(scores, r.score)
    assert np.array_equal(status, r.status)
    if score_only:
        return
    for i in range(n):
        got = ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode()
        want = r.cigar(i)
        if status[i] != 0:
            # e.g. BiWFA whose heuristic-cut searches end far past the
            # recovery score: WF_STATUS_UNATTAINABLE, no CIGAR, in both
            assert got == want == "", i
            continue
        assert O.check_cigar(got, b.pattern(i), b.text(i)), i
        if O.check_cigar(want, b.pattern(i), b.text(i)):
            assert got == want, i
        else:
            assert O.rescore(got, pen) == int(scores[i]), i


def test_default_attributes_are_served(gpu_available, wfa, oracle_mod):
    """An aligner built from an unmodified copy of wavefront_aligner_attr_default
    (wf-adaptive 10,50,1) aligns on the GPU as the reference would."""
    W, O = wfa, oracle_mod
    attr = W.default_attributes()
    h = attr.heuristic
    assert (h.strategy, h.min_wavefront_length, h.max_distance_threshold,
            h.steps_between_cutoffs) == (W.WF_HEURISTIC_WFADAPTIVE, 10, 50, 1)
    wf = W.lib().wavefront_aligner_new(attr)
    assert wf and wf.contents.engine
    p = W.generate(1, 20, first=77)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, O.Penalties(), wfadaptive=(10, 50, 1))
    for i in range(p.n):
        P, T = p.pattern(i), p.text(i)
        st = W.lib().wavefront_align(wf, P, len(P), T, len(T))
        cg = wf.contents.cigar.contents
        ops = bytes(cg.operations[cg.begin_offset:cg.end_offset]).decode()
        assert (st, cg.score, ops) == (int(r.status[i]), int(r.score[i]), r.cigar(i)), i
    W.lib().wavefront_aligner_delete(wf)

"""The pooled back-trace store of the batched path.

Pairs whose choice bytes outgrow a first-pass warp's 1 MB slice are re-run
with their choice bytes in a shared device block pool: a pair takes blocks as
its back-trace grows and returns them when done.  A pair that finds the pool
empty is retried by a later pass; the last pass runs few enough warps that all
of them can hold their largest back-trace at once.  So results must not depend
on the pool's size or on which pairs ran beside each other: only a pair whose
back-trace exceeds the whole pool reports WF_STATUS_OOM.

Integer work: scores, statuses and CIGARs are compared exactly with the CPU
checker (wavefront/wavefront_align.c:100-180 via the oracle)."""
import os

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def _mixed(W):
    """8 kbp pairs at 20 % divergence (back-traces of roughly 10-60 MB) between
    1.5 kbp pairs at 5 % (well under 1 MB, done by the first pass)."""
    big = W.generate(5, 6, first=11, param=8000, param2=200)
    small = W.generate(5, 6, first=40, param=1500, param2=50)
    pats, txts = [], []
    for i in range(6):
        pats += [big.pattern(i), small.pattern(i)]
        txts += [big.text(i), small.text(i)]
    return pats, txts


def _run(W, cfg, pats, txts, env):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        seqs, po, pl, to, tl = helpers.pack(pats, txts)
        al = W.Aligner(cfg)
        rc, scores, status, ops, ops_len, ops_off = al.align_batch(seqs, po, pl, to, tl)
        al.close()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    assert rc == 0
    return [(int(status[i]), int(scores[i]),
             ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode()) for i in range(len(pats))]


@pytest.mark.parametrize("metric", ["affine", "affine2p"])
def test_pool_results_do_not_depend_on_pool_size(gpu_available, wfa, oracle_mod, metric):
    W, O = wfa, oracle_mod
    pats, txts = _mixed(W)
    m = W.GAP_AFFINE if metric == "affine" else W.GAP_AFFINE_2P
    cfg = W.Config(metric=m)
    pen = O.Penalties(metric=m)
    b = O.PairBatch.from_lists(pats, txts)
    r = O.align(b, pen)
    want = [(int(r.status[i]), int(r.score[i]), r.cigar(i)) for i in range(len(pats))]

    # default pool: everything fits
    assert _run(W, cfg, pats, txts, {}) == want
    # 96 MB pool fed to 12 pairs of 8 MB: pass 2 runs dry, later passes finish
    assert _run(W, cfg, pats, txts, {"WF2G_POOL_MB": 96, "WF2G_POOL_PAIR_MB": 8}) == want
    # a pool of two 1 MB blocks: the large pairs report WF_STATUS_OOM, the
    # small ones (first pass, no pool) are exact
    tiny = _run(W, cfg, pats, txts, {"WF2G_POOL_MB": 2})
    for i, (got, exp) in enumerate(zip(tiny, want)):
        if i % 2:
            assert got == exp, i
        else:
            assert got == (W.WF_STATUS_OOM, 0, ""), i

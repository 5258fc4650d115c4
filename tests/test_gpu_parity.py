"""GPU parity: the sm_103a path, driven through the C ABI, against the CPU
checker and the reference's golden vectors.  Integer work: bit-exact scores,
byte-identical CIGARs, every CIGAR replayed and rescored."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

UT = helpers.utest_expected()
SY = helpers.synthetic_expected()


def cfg_of(W, spec, score_only=False, memory_mode=0, max_steps=0, wfadaptive=None):
    m, match, x, o1, e1, o2, e2 = spec
    return W.Config(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                    gap_opening2=o2, gap_extension2=e2, score_only=score_only,
                    memory_mode=memory_mode, max_steps=max_steps,
                    wfadaptive=tuple(wfadaptive) if wfadaptive else None)


HEUR = UT.get("heuristics", {})


def pen_of(O, spec):
    m, match, x, o1, e1, o2, e2 = spec
    return O.Penalties(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                       gap_opening2=o2, gap_extension2=e2)


def run_batch(W, cfg, batch):
    seqs, p_off, p_len, t_off, t_len = batch
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(seqs, p_off, p_len, t_off, t_len)
    assert rc == 0
    cig = None
    if not cfg.score_only:
        cig = [ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode() for i in range(len(p_len))]
    launches = al.launches
    al.close()
    assert launches >= 1
    return scores, status, cig


def _split_key(key):
    for mp in sorted(UT["modes"], key=len, reverse=True):
        if key.startswith(mp + "."):
            return mp, key[len(mp) + 1:]
    raise KeyError(key)


# test.biwfa.* keys run the BiWFA path (ultralow memory mode): its CIGARs
# break ties differently from the unidirectional ones, as the reference's do
@pytest.mark.parametrize("key", sorted(UT["expected"].keys()))
def test_gpu_matches_reference_goldens(gpu_available, wfa, oracle_mod, key):
    W, O = wfa, oracle_mod
    prefix, name = _split_key(key)
    mode, score_only = UT["modes"][prefix]
    spec = UT["penalty_sets"][name]
    pats, txts = helpers.utest_pairs()
    batch = helpers.pack(pats, txts)
    scores, status, cig = run_batch(W, cfg_of(W, spec, score_only, mode, 0, HEUR.get(name)),
                                    batch)
    assert (status == 0).all()
    exp = UT["expected"][key]
    pen = pen_of(O, spec)
    bad = []
    for i in range(len(pats)):
        if score_only:
            got = [int(scores[i]), helpers.crc("-")]
        else:
            assert O.check_cigar(cig[i], pats[i], txts[i]), (key, i)
            assert O.rescore(cig[i], pen) == int(scores[i]), (key, i)
            got = [O.rescore(cig[i], pen), helpers.crc(helpers.rle(cig[i]))]
        if got != exp[i]:
            bad.append(i)
    assert not bad, f"{key}: {len(bad)} pairs differ, first {bad[:5]}"


@pytest.mark.parametrize("name", sorted(SY.keys()))
def test_gpu_matches_reference_on_synthetic(gpu_available, wfa, name):
    W = wfa
    fx = SY[name]
    spec = UT["penalty_sets"][fx["penalties"]]
    p = W.generate(fx["workload"], fx["n"], param=fx["param"], param2=fx["param2"])
    batch = (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    cfg = cfg_of(W, spec, fx["score_only"], fx["memory_mode"], fx.get("max_steps", 0),
                 HEUR.get(fx["penalties"]))
    scores, status, cig = run_batch(W, cfg, batch)
    for i, (score, st, c) in enumerate(fx["rows"]):
        assert int(scores[i]) == score and int(status[i]) == st, (name, i)
        if cig is not None:
            assert helpers.crc(cig[i]) == c, (name, i)


@pytest.mark.parametrize("workload,n,spec_name,score_only", [
    (0, 3000, "affine", False),
    (1, 400, "affine", False),
    (1, 400, "affine", True),
    (2, 24, "affine2p", False),
    (1, 200, "affine.p4", False),
    (1, 200, "affine2p", True),
])
def test_gpu_matches_oracle(gpu_available, wfa, oracle_mod, workload, n, spec_name, score_only):
    W, O = wfa, oracle_mod
    spec = UT["penalty_sets"][spec_name]
    p = W.generate(workload, n, first=10_000)
    scores, status, cig = run_batch(W, cfg_of(W, spec, score_only),
                                    (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len))
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, pen_of(O, spec), score_only=score_only)
    assert np.array_equal(scores, r.score)
    assert np.array_equal(status, r.status)
    if cig is not None:
        for i in range(n):
            assert cig[i] == r.cigar(i), i


def test_gpu_edge_cases(gpu_available, wfa, oracle_mod):
    W, O = wfa, oracle_mod
    pats = [b"", b"A", b"", b"ACGT", b"ACGT" * 10, b"AAAA", b"A" * 700, b"ACGT" * 400]
    txts = [b"", b"", b"ACG", b"ACGT", b"ACGT" * 10, b"TTTT", b"C" * 3, b"ACGA" * 100]
    r = O.align(O.PairBatch.from_lists(pats, txts), O.Penalties())
    scores, status, cig = run_batch(W, W.Config(), helpers.pack(pats, txts))
    assert list(scores) == list(r.score)
    assert cig == [r.cigar(i) for i in range(len(pats))]


def test_gpu_non_acgt_bytes(gpu_available, wfa, oracle_mod):
    """Bytes outside ACGT compare as bytes (N==N matches), as in the reference."""
    W, O = wfa, oracle_mod
    pats = [b"ACGTNNNNACGT", b"acgtACGT", b"NNNN" * 50, b"ACGTRYKM" * 30]
    txts = [b"ACGTNNNACGTT", b"ACGTacgt", b"NNNA" * 50, b"ACGTRYKN" * 29]
    r = O.align(O.PairBatch.from_lists(pats, txts), O.Penalties())
    scores, status, cig = run_batch(W, W.Config(), helpers.pack(pats, txts))
    assert list(scores) == list(r.score)
    assert cig == [r.cigar(i) for i in range(len(pats))]


def test_gpu_max_steps(gpu_available, wfa, oracle_mod):
    W, O = wfa, oracle_mod
    p = W.generate(1, 64, first=777)
    r = O.align(O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len), O.Penalties(),
                max_steps=100)
    scores, status, _ = run_batch(W, W.Config(max_steps=100),
                                  (p.seqs, p.p_off, p.p_len, p.t_off, p.t_len))
    assert np.array_equal(status, r.status) and np.array_equal(scores, r.score)
    assert (status == -100).any() and (status == 0).any()


def test_drop_in_per_pair_api(gpu_available, wfa, oracle_mod):
    """wavefront_align() per pair equals the batch call and the checker."""
    W, O = wfa, oracle_mod
    p = W.generate(1, 40, first=31)
    r = O.align(O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len), O.Penalties())
    al = W.Aligner(W.Config())
    for i in range(p.n):
        st, score, ops = al.align(p.pattern(i), p.text(i))
        assert st == 0 and score == int(r.score[i]) and ops == r.cigar(i), i
    al.close()
    so = W.Aligner(W.Config(score_only=True))
    for i in range(p.n):
        st, score, ops = so.align(p.pattern(i), p.text(i))
        assert st == 0 and score == int(r.score[i]) and ops == ""
    so.close()


def test_packed2bits_entry_point(gpu_available, wfa):
    W = wfa
    enc = {ord("A"): 0, ord("C"): 1, ord("G"): 2, ord("T"): 3}

    def pack2(s):
        out = bytearray((len(s) + 3) // 4)
        for i, c in enumerate(s):
            out[i >> 2] |= enc[c] << (2 * (i & 3))
        return bytes(out)

    p = W.generate(1, 10, first=5)
    al = W.Aligner(W.Config())
    for i in range(p.n):
        a = al.align(p.pattern(i), p.text(i))
        b = al.align_packed2bits(pack2(p.pattern(i)), len(p.pattern(i)), pack2(p.text(i)),
                                 len(p.text(i)))
        assert a == b
    al.close()


def test_unsupported_configurations_fail_loudly(gpu_available, wfa):
    """No silent CPU or heuristic fallback: out-of-scope forms (here BiWFA with
    z-drop, which its breakpoint searches do not compute) return
    WF_STATUS_UNATTAINABLE (per pair) / WF2G_ERR_CONFIG (batch)."""
    W = wfa
    al = W.Aligner(W.Config(memory_mode=W.MEM_ULTRALOW))
    W.lib().wavefront_aligner_set_heuristic_zdrop(al._h, 100, 1)
    st, _, _ = al.align(b"ACGT", b"ACGA")
    assert st == W.WF_STATUS_UNATTAINABLE
    seqs, po, pl, to, tl = helpers.pack([b"ACGT"], [b"ACGA"])
    rc = al.align_batch(seqs, po, pl, to, tl)[0]
    assert rc == -2
    W.lib().wavefront_aligner_set_heuristic_none(al._h)
    st, score, ops = al.align(b"ACGT", b"ACGA")
    assert st == 0 and score == -4 and ops == "MMMX"
    al.close()


def test_drop_in_long_affine2p_pairs(gpu_available, wfa, oracle_mod):
    """wavefront_align() one pair at a time on 5-10 kbp gap-affine-2p pairs
    (whose back-traces take tens of MB) gives the batch call's results, which
    are the checker's: a single-pair call must not report WF_STATUS_OOM where
    the batch completes."""
    W, O = wfa, oracle_mod
    p = W.generate(2, 40, first=0)
    cfg = W.Config(metric=W.GAP_AFFINE_2P)
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len,
                                                               p.t_off, p.t_len)
    assert rc == 0 and (status == 0).all()
    for i in range(p.n):
        st, score, cig = al.align(p.pattern(i), p.text(i))
        assert (st, score) == (0, int(scores[i])), i
        assert cig == ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode(), i
    al.close()
    idx = [9, 17]  # two of the longest pairs of the sample
    b = O.PairBatch.from_lists([p.pattern(i) for i in idx], [p.text(i) for i in idx])
    r = O.align(b, O.Penalties(metric=4), nthreads=8)
    for j, i in enumerate(idx):
        assert int(r.score[j]) == int(scores[i]), i


def test_host_batch_in_chunks(gpu_available, wfa, oracle_mod):
    """A host batch large enough for several chunks (copies in and out on
    their own streams, kernels on two engines in turn) gives the checker's
    scores, statuses and CIGARs for every pair."""
    W, O = wfa, oracle_mod
    p = W.generate(0, 40000, first=900)
    al = W.Aligner(W.Config())
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(p.seqs, p.p_off, p.p_len,
                                                               p.t_off, p.t_len)
    al.close()
    assert rc == 0
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, O.Penalties(), nthreads=8)
    res = O.compare(b, O.Penalties(), scores, status, ops, ops_off, ops_len, r)
    assert all(res[k] == 0 for k in ("score_mismatch", "status_mismatch", "cigar_mismatch",
                                      "cigar_invalid", "rescore_mismatch")), res

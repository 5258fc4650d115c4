"""The CPU checker against the reference's own golden vectors (CPU only).

Pins the C restatement (oracle/wfa_oracle.c) to
  * every in-scope golden file of the reference test-suite
    (tests/wfa.utest.check/*.alg via tests/golden/utest_expected.json), and
  * outputs of the reference library itself on seeded synthetic pairs
    (tests/golden/synthetic_expected.json), and in the ends-free and
    extension forms (tests/golden/endsfree_expected.json: score, status,
    CIGAR and end position; the reference built with its portable extension
    kernels), and under the heuristics other than wf-adaptive
    (tests/golden/heuristics_expected.json).
"""
import numpy as np
import pytest

import helpers


def _pen(O, spec):
    m, match, x, o1, e1, o2, e2 = spec
    return O.Penalties(metric=m, match=match, mismatch=x, gap_opening1=o1, gap_extension1=e1,
                       gap_opening2=o2, gap_extension2=e2)


UT = helpers.utest_expected()


@pytest.mark.parametrize("key", sorted(UT["expected"].keys()))
def test_oracle_matches_reference_goldens(oracle_mod, key):
    O = oracle_mod
    prefix, name = key.split(".", 1) if key.startswith("test.") is False else (None, None)
    # key = "<mode prefix>.<penalty set>", mode prefixes contain dots
    for mp in sorted(UT["modes"], key=len, reverse=True):
        if key.startswith(mp + "."):
            prefix, name = mp, key[len(mp) + 1:]
            break
    mode, score_only = UT["modes"][prefix]
    pen = _pen(O, UT["penalty_sets"][name])
    pats, txts = helpers.utest_pairs()
    b = O.PairBatch.from_lists(pats, txts)
    r = O.align(b, pen, memory_mode=mode, score_only=score_only,
                wfadaptive=UT.get("heuristics", {}).get(name))
    exp = UT["expected"][key]
    assert len(exp) == b.n
    bad = []
    for i in range(b.n):
        if score_only:
            got = [int(r.score[i]), helpers.crc("-")]
        else:
            ops = r.cigar(i)
            got = [O.rescore(ops, pen), helpers.crc(helpers.rle(ops))]
            assert O.check_cigar(ops, b.pattern(i), b.text(i))
        if got != exp[i]:
            bad.append(i)
    assert not bad, f"{key}: {len(bad)} pairs differ, first {bad[:5]}"


SY = helpers.synthetic_expected()


@pytest.mark.parametrize("name", sorted(SY.keys()))
def test_oracle_matches_reference_on_synthetic(oracle_mod, wfa, name):
    O, W = oracle_mod, wfa
    fx = SY[name]
    pen = _pen(O, UT["penalty_sets"][fx["penalties"]])
    p = W.generate(fx["workload"], fx["n"], param=fx["param"], param2=fx["param2"])
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, pen, memory_mode=fx["memory_mode"], score_only=fx["score_only"],
                max_steps=fx.get("max_steps", 0),
                wfadaptive=UT.get("heuristics", {}).get(fx["penalties"]))
    for i, (score, status, c) in enumerate(fx["rows"]):
        assert int(r.score[i]) == score and int(r.status[i]) == status, (name, i)
        assert helpers.crc(r.cigar(i)) == c, (name, i)


EF = helpers.endsfree_expected()


@pytest.mark.parametrize("name", sorted(EF.keys()))
def test_oracle_matches_reference_endsfree(oracle_mod, wfa, name):
    O, W = oracle_mod, wfa
    fx = EF[name]
    pen = _pen(O, UT["penalty_sets"][fx["penalties"]])
    p = W.generate(fx["workload"], fx["n"], param=fx["param"], param2=fx["param2"])
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    r = O.align(b, pen, score_only=fx["score_only"], form=fx["form"], wfadaptive=fx["wfadaptive"])
    for i, (score, status, c, ev, eh) in enumerate(fx["rows"]):
        got = (int(r.score[i]), int(r.status[i]), helpers.crc(r.cigar(i)), int(r.end[i][0]),
               int(r.end[i][1]))
        assert got == (score, status, c, ev, eh), (name, i)
        if status in (0, 1) and not fx["score_only"] and r.cigar(i):
            # an ends-free CIGAR still spans both sequences (free ends as I/D);
            # a trimmed extension CIGAR spans the prefixes up to its end (an
            # untrimmed one -- edit, indel -- has no end position)
            if fx["form"] == "extension" and ev >= 0:
                assert O.check_cigar(r.cigar(i), b.pattern(i)[:ev], b.text(i)[:eh]), (name, i)
            else:
                assert O.check_cigar(r.cigar(i), b.pattern(i), b.text(i)), (name, i)


HX = helpers.heuristics_expected()


@pytest.mark.parametrize("name", sorted(HX.keys()))
def test_oracle_matches_reference_heuristics(oracle_mod, wfa, name):
    """Banded static/adaptive, wfmash, x-drop, z-drop and combinations
    (wavefront/wavefront_heuristic.c:229-563): score, status, CIGAR and end
    position equal the reference's, including the back-traces that read a
    wavefront a cut emptied."""
    O, W = oracle_mod, wfa
    fx = HX[name]
    pen = _pen(O, UT["penalty_sets"][fx["penalties"]])
    b = helpers.heuristic_pairs(O, W, fx)
    r = O.align(b, pen, score_only=fx["score_only"], form=fx["form"],
                heuristic=O.Heuristic(**fx["heuristic"]), memory_mode=fx.get("memory_mode", 0),
                max_steps=fx.get("max_steps", 0))
    assert len(fx["rows"]) == b.n
    for i, (score, status, c, ev, eh) in enumerate(fx["rows"]):
        got = (int(r.score[i]), int(r.status[i]), helpers.crc(r.cigar(i)), int(r.end[i][0]),
               int(r.end[i][1]))
        assert got == (score, status, c, ev, eh), (name, i)


def test_oracle_heuristic_rejections(oracle_mod, wfa):
    """Drops with edit/indel (the reference exits, wavefront/wavefront_align.c:
    83-89) and BiWFA with z-drop fail loudly."""
    O, W = oracle_mod, wfa
    p = W.generate(1, 4, first=3)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    for metric in (O.EDIT, O.INDEL):
        for st in (O.HS_XDROP, O.HS_ZDROP):
            with pytest.raises(ValueError):
                O.align(b, O.Penalties(metric), heuristic=O.Heuristic(st, xdrop=10, zdrop=10))
    with pytest.raises(ValueError):
        O.align(b, O.Penalties(), memory_mode=O.MEM_ULTRALOW,
                heuristic=O.Heuristic(O.HS_ZDROP, zdrop=50))
    O.align(b, O.Penalties(), memory_mode=O.MEM_ULTRALOW,
            heuristic=O.Heuristic(O.HS_WFADAPTIVE, 10, 50, 1))


def test_oracle_endsfree_rejections(oracle_mod, wfa):
    """Forms the restatement does not serve fail loudly: BiWFA with any
    ends-free form (the reference exits, wavefront/wavefront_align.c:67-82) and
    edit/indel with begin-free lengths and a full alignment (the reference's
    back-trace reads the begin-free diagonals as sourceless).  Their
    score-only form, and begin-free lengths with match < 0 (re-entry at
    multiples of -match, wavefront/wavefront_compute.c:124-262), are served
    and pinned to the ends-free fixtures."""
    O, W = oracle_mod, wfa
    p = W.generate(1, 4, first=3)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    with pytest.raises(ValueError):
        O.align(b, O.Penalties(), memory_mode=O.MEM_ULTRALOW, form=(5, 5, 5, 5))
    with pytest.raises(ValueError):
        O.align(b, O.Penalties(O.EDIT), form=(5, 0, 0, 0))
    with pytest.raises(ValueError):
        O.align(b, O.Penalties(O.INDEL), form=(0, 0, 5, 0))
    O.align(b, O.Penalties(O.EDIT), form=(5, 0, 0, 0), score_only=True)
    O.align(b, O.Penalties(O.INDEL), form=(0, 0, 5, 0), score_only=True)
    O.align(b, O.Penalties(match=-1), form=(5, 0, 0, 0))
    O.align(b, O.Penalties(match=-1), form=(0, 5, 0, 5))
    O.align(b, O.Penalties(match=-1), form="extension")


def test_oracle_rescoring_and_replay(oracle_mod, wfa):
    """Every CIGAR replays against its pair and rescoring gives cigar->score."""
    O, W = oracle_mod, wfa
    p = W.generate(1, 200)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    pen = O.Penalties()
    r = O.align(b, pen)
    for i in range(b.n):
        ops = r.cigar(i)
        assert O.check_cigar(ops, b.pattern(i), b.text(i))
        assert O.rescore(ops, pen) == int(r.score[i])


def test_oracle_edge_cases(oracle_mod):
    O = oracle_mod
    pats = [b"", b"A", b"", b"ACGT", b"ACGT" * 10, b"AAAA"]
    txts = [b"", b"", b"ACG", b"ACGT", b"ACGT" * 10, b"TTTT"]
    b = O.PairBatch.from_lists(pats, txts)
    r = O.align(b, O.Penalties())
    assert list(r.score) == [0, -8, -12, 0, 0, -16]
    assert [r.cigar(i) for i in range(b.n)] == ["", "D", "III", "MMMM", "M" * 40, "XXXX"]
    rs = O.align(b, O.Penalties(), max_steps=5)
    assert int(rs.status[5]) == -100 and int(rs.score[5]) == -5


def _mixed_pairs(O, seed, n):
    """Seeded pairs of four kinds: similar, a similar prefix then an unrelated
    tail, one long indel, unrelated."""
    import random
    rng = random.Random(seed)

    def mutate(s, rate):
        out = []
        for c in s:
            r = rng.random()
            if r < rate / 3:
                out.append(rng.choice("ACGT"))
            elif r < 2 * rate / 3:
                pass
            elif r < rate:
                out += [c, rng.choice("ACGT")]
            else:
                out.append(c)
        return "".join(out)

    pats, txts = [], []
    for i in range(n):
        length = rng.randint(50, 700)
        p = "".join(rng.choice("ACGT") for _ in range(length))
        kind = i % 4
        if kind == 0:
            t = mutate(p, rng.uniform(0, 0.2))
        elif kind == 1:
            cut = rng.randint(length // 4, length)
            t = mutate(p[:cut], 0.05) + "".join(rng.choice("ACGT") for _ in range(rng.randint(0, length)))
        elif kind == 2:
            a = rng.randint(0, length)
            t = mutate(p[:a] + p[min(length, a + rng.randint(10, 150)):], 0.03)
        else:
            t = "".join(rng.choice("ACGT") for _ in range(rng.randint(0, 300)))
        pats.append(p.encode())
        txts.append(t.encode())
    return O.PairBatch.from_lists(pats, txts)


def test_oracle_flags(oracle_mod, wfa):
    """The checker marks the pairs its GPU comparison leaves out: back-traces
    through a wavefront a cut emptied (common under a wide x-drop on unrelated
    sequences, absent on the generator's workloads) and runs past the
    reference's per-pair wavefront table (x-drop with match 0)."""
    O, W = oracle_mod, wfa
    mixed = _mixed_pairs(O, 1, 200)
    r = O.align(mixed, O.Penalties(), heuristic=O.Heuristic(O.HS_XDROP, xdrop=100,
                                                            steps_between_cutoffs=2))
    assert ((r.flags & O.FLAG_STALE_SOURCE) > 0).sum() > 50
    assert ((r.flags & O.FLAG_OVER_BOUND) > 0).sum() > 10
    r = O.align(mixed, O.Penalties(), heuristic=O.Heuristic(O.HS_WFADAPTIVE, 10, 50, 1))
    assert not (r.flags & O.FLAG_OVER_BOUND).any()
    for wl in (1, 6):
        p = W.generate(wl, 120)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        r = O.align(b, O.Penalties(O.GAP_AFFINE, -2, 3, 1, 4),
                    heuristic=O.Heuristic(O.HS_XDROP, xdrop=80, steps_between_cutoffs=1))
        assert not r.flags.any()

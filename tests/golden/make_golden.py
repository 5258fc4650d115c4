"""Regenerates the golden fixtures under tests/golden/ (run where the reference
sources are available; the fixtures themselves travel with the repo).

1. ``utest.seq.gz`` -- the reference test-suite's 305 input pairs
   (tests/wfa.utest.seq of smarco/WFA2-lib), gzipped.
2. ``utest_expected.json`` -- for every in-scope configuration of the
   reference test-suite (tests/wfa.utest.sh:35-64: gap-affine, gap-affine-2p
   and penalty sets p0..p5; modes full CIGAR/high, score-only, med, BiWFA
   full CIGAR and BiWFA score-only), the reference's own expected output per pair from
   tests/wfa.utest.check/*.alg: the printed score and the CRC32 of the
   printed RLE CIGAR ("-" when there is none).
3. ``synthetic_expected.json`` -- outputs of the UNMODIFIED reference library
   (oracle/_ref/libwfa_ref.so, built from the reference sources by
   oracle/Makefile) on seeded synthetic pairs of each workload shape
   (wfa2-lib_gb300/csrc/wfa_datagen.c): cigar->score and CRC32 of the
   operations string per pair.
4. ``endsfree_expected.json`` -- the same for the ends-free and extension
   forms (wavefront/wavefront_attributes.h:55-69), from the reference built
   without host tuning (oracle/_ref/libwfa_ref_scalar.so: its portable
   extension kernels, as on aarch64), with cigar->end_v / end_h per pair.
5. ``heuristics_expected.json`` -- the same for the heuristics other than
   wf-adaptive (wavefront/wavefront_heuristic.c: banded static and adaptive,
   wfmash, x-drop, z-drop and combinations).  Pairs the reference cannot
   finish are left out, found first with the CPU restatement: those that run
   past its per-pair wavefront table (it exits, wavefront/wavefront_compute.c:
   442-446) and, for edit/indel, those a cut leaves unable to reach the end
   (it faults in alignment scope and loops in score-only scope).  Each set
   lists the pair indices it keeps.

Usage:  python tests/golden/make_golden.py [/path/to/WFA2-lib] [--only=endsfree|heuristics]
"""
import gzip
import json
import os
import sys
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "wfa2-lib_gb300"))

# name -> (metric, match, mismatch, o1, e1, o2, e2); tests/wfa.utest.sh:47-57
PENALTY_SETS = {
    "affine": (3, 0, 4, 6, 2, 24, 1),
    "affine2p": (4, 0, 4, 6, 2, 24, 1),
    "affine.p0": (3, 0, 1, 2, 1, 24, 1),
    "affine.p1": (3, 0, 3, 1, 4, 24, 1),
    "affine.p2": (3, 0, 5, 3, 2, 24, 1),
    "affine.p3": (3, -5, 1, 2, 1, 24, 1),
    "affine.p4": (3, -2, 3, 1, 4, 24, 1),
    "affine.p5": (3, -3, 5, 3, 2, 24, 1),
    "affine.wfapt0": (3, 0, 4, 6, 2, 24, 1),
    "affine.wfapt1": (3, 0, 4, 6, 2, 24, 1),
    "edit": (1, 0, 0, 0, 0, 0, 0),
    "indel": (0, 0, 0, 0, 0, 0, 0),
}
# penalty sets with no golden file of the reference test-suite (gap-linear:
# the indel penalty sits in the gap_opening1 slot)
EXTRA_SETS = {
    "linear": (2, 0, 4, 2, 0, 0, 0),
    "linear.m1": (2, -1, 3, 2, 0, 0, 0),
}
# wf-adaptive heuristic of a penalty set: (min_wavefront_length,
# max_distance_threshold, steps_between_cutoffs); tests/wfa.utest.sh:61-63
HEURISTICS = {
    "affine.wfapt0": (10, 50, 1),
    "affine.wfapt1": (10, 50, 10),
}
# file prefix -> (memory mode, score only); tests/wfa.utest.sh:35-40
MODES = {
    "test": (0, False),
    "test.score": (0, True),
    "test.pb": (1, False),
    "test.biwfa.score": (3, True),
    "test.biwfa": (3, False),
}
# synthetic fixture sets:
# name -> (workload, n, penalty set, score_only, memory mode, param, param2[, max_steps])
SYNTHETIC = {
    "w0_affine_full": (0, 2000, "affine", False, 0, 0, 0),
    "w0_affine_score": (0, 2000, "affine", True, 0, 0, 0),
    "w1_affine_full": (1, 300, "affine", False, 0, 0, 0),
    "w1_affine_score": (1, 300, "affine", True, 0, 0, 0),
    "w2_affine2p_full": (2, 40, "affine2p", False, 0, 0, 0),
    "w5_affine_p3_full": (5, 300, "affine.p3", False, 0, 400, 80),
    # BiWFA (ultralow memory mode) on pairs long enough to split at breakpoints
    "w5_affine_biwfa_full": (5, 60, "affine", False, 3, 3000, 300),
    "w5_affine2p_biwfa_full": (5, 30, "affine2p", False, 3, 3000, 300),
    "w5_affine_p3_biwfa_full": (5, 30, "affine.p3", False, 3, 3000, 300),
    "w1_affine_biwfa_score": (1, 100, "affine", True, 3, 0, 0),
    # 100 kbp pairs at 10-15 % divergence: nine levels of breakpoints
    "w3_affine_biwfa_full": (3, 2, "affine", False, 3, 0, 0),
    # max_alignment_steps inside the breakpoint search and inside base cases
    "w5_affine_biwfa_ms700": (5, 40, "affine", False, 3, 3000, 300, 700),
    "w0_affine_biwfa_ms12": (0, 200, "affine", False, 3, 0, 0, 12),
    "w1_affine_biwfa_ms300_score": (1, 100, "affine", True, 3, 0, 0, 300),
    # the wf-adaptive heuristic (the reference's default attributes)
    "w1_wfapt0_full": (1, 300, "affine.wfapt0", False, 0, 0, 0),
    "w4_wfapt0_full": (4, 60, "affine.wfapt0", False, 0, 0, 0),
    "w1_wfapt1_score": (1, 300, "affine.wfapt1", True, 0, 0, 0),
    "w5_wfapt0_biwfa_full": (5, 40, "affine.wfapt0", False, 3, 3000, 300),
    "w1_edit_full": (1, 300, "edit", False, 0, 0, 0),
    "w1_indel_full": (1, 300, "indel", False, 0, 0, 0),
    "w1_linear_full": (1, 300, "linear", False, 0, 0, 0),
    "w1_linear_score": (1, 300, "linear", True, 0, 0, 0),
    "w5_linear_m1_full": (5, 60, "linear.m1", False, 0, 2000, 150),
    "w6_edit_prune_full": (6, 12, "edit", False, 0, 3000, 200),
    "w6_edit_prune_score": (6, 12, "edit", True, 0, 3000, 200),
    "w5_indel_score": (5, 40, "indel", True, 0, 2000, 100),
    "w1_edit_ms50": (1, 100, "edit", False, 0, 0, 0, 50),
    "w5_edit_biwfa_full": (5, 20, "edit", False, 3, 3000, 200),
    "w6_edit_biwfa_full": (6, 8, "edit", False, 3, 3000, 150),
    "w1_linear_biwfa_full": (1, 100, "linear", False, 3, 0, 0),
    "w5_indel_biwfa_score": (5, 20, "indel", True, 3, 3000, 200),
}

# name: (workload, n, penalties, score_only, param, param2, form, wf-adaptive)
# form: (pattern_begin_free, pattern_end_free, text_begin_free, text_end_free)
# or "extension"
ENDSFREE = {
    "w1_affine_ef5": (1, 300, "affine", False, 0, 0, (5, 5, 5, 5), None),
    "w1_affine_ef_text": (1, 300, "affine", False, 0, 0, (0, 0, 200, 200), None),
    "w1_affine_ef_pattern": (1, 300, "affine", False, 0, 0, (150, 150, 0, 0), None),
    "w1_affine_ef_score": (1, 300, "affine", True, 0, 0, (50, 50, 50, 50), None),
    "w1_affine_ext": (1, 300, "affine", False, 0, 0, "extension", None),
    "w1_affine2p_ext": (1, 200, "affine2p", False, 0, 0, "extension", None),
    "w5_affine2p_ef": (5, 100, "affine2p", False, 300, 150, (30, 0, 0, 30), None),
    "w5_affine2p_ext_div": (5, 100, "affine2p", False, 120, 300, "extension", None),
    "w5_affine_p3_ext": (5, 100, "affine.p3", False, 300, 150, "extension", None),
    "w5_affine_p3_endonly": (5, 100, "affine.p3", False, 300, 150, (0, 40, 0, 40), None),
    "w1_wfapt0_ef": (1, 200, "affine.wfapt0", False, 0, 0, (10, 10, 10, 10), (10, 50, 1)),
    "w0_affine_ef_bounds": (0, 100, "affine", False, 0, 0, (99, 99, 99, 99), None),
    "w1_edit_ext": (1, 200, "edit", False, 0, 0, "extension", None),
    "w1_linear_ef": (1, 200, "linear", False, 0, 0, (20, 20, 20, 20), None),
    "w1_linear_ext": (1, 200, "linear.m1", False, 0, 0, "extension", None),
    "w5_indel_endonly": (5, 60, "indel", False, 500, 100, (0, 40, 0, 40), None),
    # begin-free lengths with match < 0: the free diagonals enter at the scores
    # that are multiples of -match (wavefront/wavefront_compute.c:124-262)
    "w1_affine_p4_ef_begin": (1, 200, "affine.p4", False, 0, 0, (20, 20, 20, 20), None),
    "w1_affine_p4_ef_begin_score": (1, 200, "affine.p4", True, 0, 0, (20, 20, 20, 20), None),
    "w5_affine_p3_ef_text": (5, 100, "affine.p3", False, 300, 150, (0, 0, 60, 60), None),
    "w1_linear_m1_ef_begin": (1, 150, "linear.m1", False, 0, 0, (30, 10, 30, 10), None),
    "w1_affine_p4_ef_begin_wfapt": (1, 150, "affine.p4", False, 0, 0, (15, 15, 15, 15),
                                    (10, 50, 1)),
    # edit and indel with begin-free lengths, score only (a full alignment's
    # back-trace reads the begin-free diagonals as sourceless)
    "w1_edit_ef_begin_score": (1, 200, "edit", True, 0, 0, (20, 20, 20, 20), None),
    "w0_edit_ef_bounds_score": (0, 300, "edit", True, 0, 0, (99, 99, 99, 99), None),
    "w5_indel_ef_begin_score": (5, 60, "indel", True, 500, 100, (40, 0, 40, 0), None),
}


# heuristic strategies (wavefront/wavefront_heuristic.h:41-49) and parameters
def _h(strategy, **kw):
    return {"strategy": strategy, **kw}


BS, BA, WA, XD, ZD, WM = 0x01, 0x02, 0x04, 0x10, 0x20, 0x40
# name: (workload, n, penalties, score_only, param, param2, form, heuristic)
HEURISTIC_SETS = {
    "w1_affine_bstatic": (1, 60, "affine", False, 0, 0, None, _h(BS, min_k=-30, max_k=30)),
    "w1_affine_bstatic_score": (1, 60, "affine", True, 0, 0, None, _h(BS, min_k=-30, max_k=30)),
    "w6_affine_badapt": (6, 60, "affine", False, 0, 0, None,
                         _h(BA, min_k=-20, max_k=20, steps_between_cutoffs=1)),
    "w1_affine_badapt3_ext": (1, 60, "affine", False, 0, 0, "extension",
                              _h(BA, min_k=-20, max_k=20, steps_between_cutoffs=3)),
    "w1_affine_wfmash": (1, 60, "affine", False, 0, 0, None,
                         _h(WM, min_wavefront_length=10, max_distance_threshold=50,
                            steps_between_cutoffs=1)),
    "w6_affine_p4_xdrop": (6, 60, "affine.p4", False, 0, 0, None,
                           _h(XD, xdrop=50, steps_between_cutoffs=1)),
    "w6_affine_p3_xdrop_ext": (6, 60, "affine.p3", False, 0, 0, "extension",
                               _h(XD, xdrop=100, steps_between_cutoffs=1)),
    "w6_affine_p4_zdrop_score": (6, 60, "affine.p4", True, 0, 0, None,
                                 _h(ZD, zdrop=50, steps_between_cutoffs=1)),
    "w6_affine_p4_zdrop_full": (6, 60, "affine.p4", False, 0, 0, None,
                                _h(ZD, zdrop=50, steps_between_cutoffs=1)),
    "w6_affine_p4_zdrop_ext": (6, 60, "affine.p4", False, 0, 0, "extension",
                               _h(ZD, zdrop=50, steps_between_cutoffs=2)),
    "w6_affine_p4_wfa_xdrop": (6, 60, "affine.p4", False, 0, 0, None,
                               _h(WA | XD, min_wavefront_length=10, max_distance_threshold=50,
                                  xdrop=60, steps_between_cutoffs=1)),
    "w1_affine_xdrop_bstatic_ef": (1, 60, "affine", False, 0, 0, (20, 20, 20, 20),
                                   _h(XD | BS, xdrop=40, min_k=-30, max_k=30,
                                      steps_between_cutoffs=1)),
    "w6_affine2p_xdrop": (6, 60, "affine2p", False, 0, 0, None,
                          _h(XD, xdrop=100, steps_between_cutoffs=1)),
    "w1_affine2p_bstatic_score": (1, 60, "affine2p", True, 0, 0, None,
                                  _h(BS, min_k=-25, max_k=25)),
    "w6_affine2p_zdrop": (6, 60, "affine2p", False, 0, 0, None,
                          _h(ZD, zdrop=100, steps_between_cutoffs=1)),
    "w1_linear_badapt": (1, 60, "linear", False, 0, 0, None,
                         _h(BA, min_k=-20, max_k=20, steps_between_cutoffs=1)),
    "w6_linear_m1_xdrop_ext": (6, 60, "linear.m1", False, 0, 0, "extension",
                               _h(XD, xdrop=60, steps_between_cutoffs=1)),
    "w1_edit_bstatic": (1, 60, "edit", False, 0, 0, None, _h(BS, min_k=-60, max_k=60)),
    "w1_edit_badapt": (1, 60, "edit", False, 0, 0, None,
                       _h(BA, min_k=-30, max_k=30, steps_between_cutoffs=1)),
    "w1_indel_wfmash_score": (1, 60, "indel", True, 0, 0, None,
                              _h(WM, min_wavefront_length=10, max_distance_threshold=50,
                                 steps_between_cutoffs=1)),
    # null inputs widen the range to diagonal 0 (wavefront/wavefront.c:110-117):
    # cases where that regrows cut cells
    "w5_affine_p4_bstatic_score_6k": (5, 16, "affine.p4", True, 6000, 300, None,
                                      _h(BS, min_k=-40, max_k=40)),
    "w1_affine2p_xdrop_full": (1, 120, "affine2p", False, 0, 0, None,
                               _h(XD, xdrop=80, steps_between_cutoffs=1)),
    "w6_affine2p_badapt_full": (6, 60, "affine2p", False, 0, 0, None,
                                _h(BA, min_k=-25, max_k=25, steps_between_cutoffs=2)),
    # BiWFA (ultralow memory, the optional ninth field): the breakpoint
    # searches take the heuristic, the base cases do not
    # (wavefront/wavefront_bialigner.c:52-71)
    "w1_affine_biwfa_bstatic": (1, 60, "affine", False, 0, 0, None,
                                _h(BS, min_k=-30, max_k=30), 3),
    "w1_affine2p_biwfa_xdrop": (1, 60, "affine2p", False, 0, 0, None,
                                _h(XD, xdrop=80, steps_between_cutoffs=1), 3),
    "w1_affine_p4_biwfa_wfmash_score": (1, 60, "affine.p4", True, 0, 0, None,
                                        _h(WM, min_wavefront_length=10, max_distance_threshold=50,
                                           steps_between_cutoffs=1), 3),
    # edit and indel whose band leaves the end outside: the null wavefronts do
    # not end the alignment (wavefront/wavefront_extend.c:93-101), the step
    # limit (the optional tenth field) does
    "w6_indel_bstatic_score_ms": (6, 20, "indel", True, 0, 0, None,
                                  _h(BS, min_k=-30, max_k=30), 0, 3000),
    "w6_edit_bstatic_ef_score_ms": (6, 20, "edit", True, 0, 0, (20, 20, 20, 20),
                                    _h(BS, min_k=-30, max_k=30), 0, 3000),
    "w1_edit_bstatic5_ms": (1, 40, "edit", False, 0, 0, None, _h(BS, min_k=-5, max_k=5), 0,
                            400),
    # ... and in BiWFA's breakpoint searches, which step on to the step limit
    "w6_edit_biwfa_bstatic_score_ms": (6, 20, "edit", True, 0, 0, None,
                                       _h(BS, min_k=-30, max_k=30), 3, 3000),
    "w1_indel_biwfa_bstatic5_ms": (1, 40, "indel", False, 0, 0, None,
                                   _h(BS, min_k=-5, max_k=5), 3, 400),
}


def heuristic_of(spec):
    """The CPU checker's Heuristic for a fixture set's heuristic dict."""
    from oracle import oracle as O
    return O.Heuristic(**spec)


def crc(s: str) -> int:
    return zlib.crc32(s.encode()) & 0xFFFFFFFF


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = [a[len("--only="):] for a in sys.argv[1:] if a.startswith("--only=")]
    if only == ["heuristics"]:
        return heuristics_fixtures()
    if only == ["endsfree"]:
        return endsfree_fixtures()
    from oracle import oracle as O
    ref = args[0] if args else O.reference_dir()
    with open(os.path.join(ref, "tests", "wfa.utest.seq"), "rb") as f:
        raw = f.read()
    with open(os.path.join(HERE, "utest.seq.gz"), "wb") as fo:
        with gzip.GzipFile(fileobj=fo, mode="wb", compresslevel=9, mtime=0) as f:
            f.write(raw)
    expected = {}
    for mode_prefix in MODES:
        for name in PENALTY_SETS:
            path = os.path.join(ref, "tests", "wfa.utest.check", f"{mode_prefix}.{name}.alg")
            rows = []
            with open(path) as f:
                for line in f:
                    line = line.rstrip("\n")
                    if not line:
                        continue
                    score, cig = line.split("\t")
                    rows.append([int(score), crc(cig)])
            expected[f"{mode_prefix}.{name}"] = rows
    with open(os.path.join(HERE, "utest_expected.json"), "w") as f:
        json.dump({"penalty_sets": {**PENALTY_SETS, **EXTRA_SETS}, "heuristics": HEURISTICS,
                   "modes": MODES, "expected": expected}, f, separators=(",", ":"))

    from oracle import oracle as O
    import wfa2gpu as W
    O.build(ref=True)
    W.build()
    synth = {}
    for name, spec in SYNTHETIC.items():
        wl, n, pset, so, mm, param, param2 = spec[:7]
        max_steps = spec[7] if len(spec) > 7 else 0
        m, mi, mm_, o1, e1, o2, e2 = {**PENALTY_SETS, **EXTRA_SETS}[pset]
        pen = O.Penalties(metric=m, match=mi, mismatch=mm_, gap_opening1=o1, gap_extension1=e1,
                          gap_opening2=o2, gap_extension2=e2)
        p = W.generate(wl, n, param=param, param2=param2)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        r = O.align(b, pen, memory_mode=mm, score_only=so, kind="reference", max_steps=max_steps,
                    wfadaptive=HEURISTICS.get(pset))
        rows = [[int(r.score[i]), int(r.status[i]), crc(r.cigar(i))] for i in range(n)]
        synth[name] = {"workload": wl, "n": n, "param": param, "param2": param2,
                       "penalties": pset, "score_only": so, "memory_mode": mm,
                       "max_steps": max_steps, "rows": rows}
        print(name, "done")
    with open(os.path.join(HERE, "synthetic_expected.json"), "w") as f:
        json.dump(synth, f, separators=(",", ":"))

    endsfree_fixtures()
    heuristics_fixtures()


def endsfree_fixtures():
    from oracle import oracle as O
    import wfa2gpu as W
    O.build(ref=True)
    W.build()
    ends = {}
    for name, (wl, n, pset, so, param, param2, form, heur) in ENDSFREE.items():
        m, mi, mm_, o1, e1, o2, e2 = {**PENALTY_SETS, **EXTRA_SETS}[pset]
        pen = O.Penalties(metric=m, match=mi, mismatch=mm_, gap_opening1=o1, gap_extension1=e1,
                          gap_opening2=o2, gap_extension2=e2)
        p = W.generate(wl, n, param=param, param2=param2)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        r = O.align(b, pen, score_only=so, kind="reference_scalar", form=form, wfadaptive=heur)
        rows = [[int(r.score[i]), int(r.status[i]), crc(r.cigar(i)), int(r.end[i][0]),
                 int(r.end[i][1])] for i in range(n)]
        ends[name] = {"workload": wl, "n": n, "param": param, "param2": param2,
                      "penalties": pset, "score_only": so, "form": form, "wfadaptive": heur,
                      "rows": rows}
        print(name, "done")
    with open(os.path.join(HERE, "endsfree_expected.json"), "w") as f:
        json.dump(ends, f, separators=(",", ":"))


def heuristics_fixtures():
    from oracle import oracle as O
    import wfa2gpu as W
    O.build(ref=True)
    W.build()
    heur = {}
    for name, spec in HEURISTIC_SETS.items():
        wl, n, pset, so, param, param2, form, hspec = spec[:8]
        mm = spec[8] if len(spec) > 8 else 0
        ms = spec[9] if len(spec) > 9 else 0
        m, mi, mm_, o1, e1, o2, e2 = {**PENALTY_SETS, **EXTRA_SETS}[pset]
        pen = O.Penalties(metric=m, match=mi, mismatch=mm_, gap_opening1=o1, gap_extension1=e1,
                          gap_opening2=o2, gap_extension2=e2)
        h = heuristic_of(hspec)
        p = W.generate(wl, n, param=param, param2=param2)
        b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
        a = O.align(b, pen, score_only=so, kind="port", form=form, heuristic=h, memory_mode=mm,
                    max_steps=ms)
        # (an edit/indel pair the checker ends as unreachable never ends in the
        # reference without a step limit: left out)
        keep = [i for i in range(n) if not (a.flags[i] & O.FLAG_OVER_BOUND)
                and not (m <= 1 and a.status[i] == 1)]
        sub = O.PairBatch.from_lists([b.pattern(i) for i in keep], [b.text(i) for i in keep])
        r = O.align(sub, pen, score_only=so, kind="reference_scalar", form=form, heuristic=h,
                    memory_mode=mm, max_steps=ms)
        rows = [[int(r.score[j]), int(r.status[j]), crc(r.cigar(j)), int(r.end[j][0]),
                 int(r.end[j][1])] for j in range(sub.n)]
        heur[name] = {"workload": wl, "n": n, "param": param, "param2": param2,
                      "penalties": pset, "score_only": so, "form": form, "heuristic": hspec,
                      "memory_mode": mm, "keep": keep, "rows": rows}
        if ms:
            heur[name]["max_steps"] = ms
        print(name, "done", len(keep), "of", n)
    with open(os.path.join(HERE, "heuristics_expected.json"), "w") as f:
        json.dump(heur, f, separators=(",", ":"))


if __name__ == "__main__":
    main()

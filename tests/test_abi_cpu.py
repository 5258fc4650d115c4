"""The C ABI without a GPU: library loads, exports what include/wfa2gpu.h
declares, keeps the reference's attribute layout and defaults, the host-side
CIGAR helpers work, and no alignment is ever computed on the CPU."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "wfa2gpu.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\(", src, re.M))
    keywords = {"int", "void", "char", "bool", "if", "while", "for", "return", "sizeof"}
    return {n for n in names if n not in keywords}


def test_library_exports_every_declared_symbol(wfa):
    lib = wfa.lib()
    decl = declared_functions() | {"wavefront_aligner_attr_default"}
    missing = [n for n in sorted(decl) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(wfa.EXPORTED) <= decl


def test_attribute_defaults_match_reference(wfa):
    a = wfa.default_attributes()
    # wavefront/wavefront_attributes.c:38-100
    assert a.distance_metric == wfa.GAP_AFFINE and a.alignment_scope == wfa.COMPUTE_ALIGNMENT
    assert (a.affine_penalties.match, a.affine_penalties.mismatch, a.affine_penalties.gap_opening,
            a.affine_penalties.gap_extension) == (0, 4, 6, 2)
    p = a.affine2p_penalties
    assert (p.match, p.mismatch, p.gap_opening1, p.gap_extension1, p.gap_opening2,
            p.gap_extension2) == (0, 4, 6, 2, 24, 1)
    assert (a.linear_penalties.mismatch, a.linear_penalties.indel) == (4, 2)
    assert a.heuristic.strategy == 4 and a.heuristic.min_wavefront_length == 10
    assert a.heuristic.max_distance_threshold == 50 and a.heuristic.steps_between_cutoffs == 1
    assert a.memory_mode == wfa.MEM_HIGH
    assert a.system.max_alignment_steps == 2**31 - 1 and a.system.max_num_threads == 1
    assert a.system.probe_interval_global == 3000 and a.system.min_offsets_per_thread == 500


def test_attribute_layout_matches_reference(wfa, oracle_mod, tmp_path):
    """Field offsets of wavefront_aligner_attr_t equal the reference's (probe
    compiled against the reference headers where they exist)."""
    ref = oracle_mod.reference_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "wavefront")):
        pytest.skip("reference headers not present on this host")
    fields = [f[0] for f in wfa.AlignerAttr._fields_]
    probe = tmp_path / "probe.c"
    probe.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "wavefront/wavefront_attributes.h"\n'
        "int main(void){\n" +
        "".join(f'printf("%zu\\n", offsetof(wavefront_aligner_attr_t,{f}));\n' for f in fields) +
        'printf("%zu\\n", sizeof(wavefront_aligner_attr_t));return 0;}\n')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I" + ref, "-o", str(exe), str(probe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    mine = [getattr(wfa.AlignerAttr, f).offset for f in fields] + [C.sizeof(wfa.AlignerAttr)]
    assert got == mine


def test_cigar_helpers_on_host(wfa, oracle_mod):
    L, O = wfa.lib(), oracle_mod
    L.cigar_new.restype = C.POINTER(wfa.Cigar)
    L.cigar_new.argtypes = [C.c_int]
    L.cigar_free.argtypes = [C.POINTER(wfa.Cigar)]
    L.cigar_sprint_SAM_CIGAR.argtypes = [C.c_char_p, C.POINTER(wfa.Cigar), C.c_bool]
    ops = "MMMXMMIIIMMDDMMMMXX"
    pat, txt = b"ACGTACGGAAACGTCC", b"ACGAACTTTGGAAAGG"
    cg = L.cigar_new(64)
    C.memmove(cg.contents.operations, ops.encode(), len(ops))
    cg.contents.begin_offset, cg.contents.end_offset = 0, len(ops)
    buf = C.create_string_buffer(256)
    L.cigar_sprint(buf, cg, True)
    assert buf.value.decode() == O.cigar_rle(ops)
    L.cigar_sprint_SAM_CIGAR(buf, cg, True)
    assert buf.value.decode() == "3=1X2=3I2=2D4=2X"
    ap = wfa.AffinePenalties(0, 4, 6, 2)
    assert L.cigar_score_gap_affine(cg, C.byref(ap)) == O.rescore_affine(ops, 0, 4, 6, 2)
    a2 = wfa.Affine2pPenalties(0, 4, 6, 2, 24, 1)
    assert L.cigar_score_gap_affine2p(cg, C.byref(a2)) == O.rescore_affine2p(ops, 0, 4, 6, 2, 24, 1)
    assert L.cigar_check_alignment(None, pat, len(pat), txt, len(txt), cg, False) == \
        O.check_cigar(ops, pat, txt)
    L.cigar_free(cg)


def test_no_cpu_fallback_without_gpu(wfa):
    """Where no GPU is visible, aligning fails loudly (no silent CPU path)."""
    if wfa.lib().wfa2gpu_device() >= 0:
        pytest.skip("a GPU is visible on this host")
    attr = wfa.Config().attributes()
    h = wfa.lib().wavefront_aligner_new(C.byref(attr))
    assert h and not h.contents.engine
    st = wfa.lib().wavefront_align(h, b"ACGT", 4, b"ACGA", 4)
    assert st == wfa.WF_STATUS_UNATTAINABLE
    z = np.zeros(1, np.int64)
    rc = wfa.lib().wavefront_align_batch(h, 1, None, None, None, None, None, None, None, None,
                                         None, None)
    assert rc == -1  # WF2G_ERR_NO_GPU
    wfa.lib().wavefront_aligner_delete(h)


def test_reference_style_caller_compiles(wfa, tmp_path):
    """A C caller written against the reference API (same includes, fields
    and calls as a reference example) compiles and links against the library."""
    src = tmp_path / "caller.c"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    str(src), "-L", os.path.dirname(wfa.LIB_PATH), "-lwfa2gpu",
                    "-Wl,-rpath," + os.path.dirname(wfa.LIB_PATH)], check=True)


CALLER = r'''
#include "utils/commons.h"
#include "wavefront/wavefront_align.h"
int main(void) {
  const char* p = "GATTACAGATTACAGGG";
  const char* t = "GATCACAGATTTACAGG";
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_affine;
  attr.affine_penalties.mismatch = 4;
  attr.affine_penalties.gap_opening = 6;
  attr.affine_penalties.gap_extension = 2;
  attr.heuristic.strategy = wf_heuristic_none;
  wavefront_aligner_t* wf = wavefront_aligner_new(&attr);
  int st = wavefront_align(wf, p, strlen(p), t, strlen(t));
  printf("%d %d\n", st, wf->cigar->score);
  cigar_print_pretty(stdout, wf->cigar, p, strlen(p), t, strlen(t));
  printf("%d\n", cigar_score_gap_affine(wf->cigar, &attr.affine_penalties));
  wavefront_aligner_delete(wf);
  return st == 0 ? 0 : 1;
}
'''


def test_heuristic_setters_add_strategies(wfa):
    """The setters add to the strategy set as the reference's do
    (wavefront/wavefront_heuristic.c:40-113); "none" clears it; one
    steps_between_cutoffs serves every strategy."""
    L = wfa.lib()
    attr = wfa.default_attributes()  # wf-adaptive (wavefront/wavefront_attributes.c:71-76)
    h = L.wavefront_aligner_new(C.byref(attr))
    assert h
    L.wavefront_aligner_set_heuristic_none.argtypes = [C.c_void_p]
    for name in ("xdrop", "zdrop"):
        getattr(L, f"wavefront_aligner_set_heuristic_{name}").argtypes = [C.c_void_p, C.c_int,
                                                                          C.c_int]
    L.wavefront_aligner_set_heuristic_banded_static.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.wavefront_aligner_set_heuristic_wfadaptive.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                                             C.c_int]
    assert h.contents.heuristic.strategy == wfa.WF_HEURISTIC_WFADAPTIVE
    L.wavefront_aligner_set_heuristic_none(h)
    assert h.contents.heuristic.strategy == 0
    L.wavefront_aligner_set_heuristic_xdrop(h, 40, 3)
    L.wavefront_aligner_set_heuristic_banded_static(h, -12, 12)
    hs = h.contents.heuristic
    assert hs.strategy == wfa.WF_HEURISTIC_XDROP | wfa.WF_HEURISTIC_BANDED_STATIC
    assert (hs.xdrop, hs.min_k, hs.max_k, hs.steps_between_cutoffs) == (40, -12, 12, 3)
    L.wavefront_aligner_set_heuristic_wfadaptive(h, 10, 50, 1)
    assert h.contents.heuristic.strategy == (wfa.WF_HEURISTIC_XDROP | wfa.WF_HEURISTIC_BANDED_STATIC
                                             | wfa.WF_HEURISTIC_WFADAPTIVE)
    assert h.contents.heuristic.steps_between_cutoffs == 1
    wfa.lib().wavefront_aligner_delete(h)


def _maxtrim_py(ops, match, x, o, e, linear=False):
    """Maximal-score prefix as alignment/cigar_utils.c:112-220 computes it."""
    earn = match if match != 0 else -1
    score = best = v = h = bv = bh = 0
    best_i, last = 0, ""
    for i, op in enumerate(ops):
        if op == "M":
            score -= earn; v += 1; h += 1
        elif op == "X":
            score -= x; v += 1; h += 1
        else:
            score -= o if linear else e + (0 if last == op else o)
            if op == "I":
                h += 1
            else:
                v += 1
        last = op
        if score > best:
            best, best_i, bv, bh = score, i, v, h
    # (the reference reports a trim when the best prefix is not the whole
    # CIGAR; a best score of 0 leaves the offset at the first operation)
    was_trimmed = best_i != len(ops) - 1
    return ((ops[:best_i + 1], best, bv, bh) if best > 0 else ("", None, -1, -1)), was_trimmed


def test_maxtrim_and_display_on_host(wfa, tmp_path):
    """cigar_maxtrim_* and wavefront_aligner_maxtrim_cigar trim to the
    maximal-score prefix (alignment/cigar_utils.c:112-318); the display calls
    print the reference's labels (wavefront/wavefront_aligner.c:680-735)."""
    L = wfa.lib()
    L.cigar_new.restype = C.POINTER(wfa.Cigar)
    L.cigar_new.argtypes = [C.c_int]
    L.cigar_free.argtypes = [C.POINTER(wfa.Cigar)]
    L.cigar_maxtrim_gap_affine.restype = C.c_bool
    L.cigar_maxtrim_gap_affine2p.restype = C.c_bool
    for ops in ["MMMXMMIIIMMDDMMMMXX", "MMMMMMMMXXXXXXXIIIIIIIIII", "XXIIDD", "MMXMDDDDDDDDMM"]:
        for match in (0, -2):
            cg = L.cigar_new(64)
            C.memmove(cg.contents.operations, ops.encode(), len(ops))
            cg.contents.begin_offset, cg.contents.end_offset = 0, len(ops)
            ap = wfa.AffinePenalties(match, 4, 6, 2)
            trimmed = L.cigar_maxtrim_gap_affine(cg, C.byref(ap))
            (want_ops, want_score, ev, eh), want_trimmed = _maxtrim_py(ops, match, 4, 6, 2)
            c = cg.contents
            got = bytes(c.operations[c.begin_offset:c.end_offset]).decode()
            assert got == want_ops, (ops, match)
            assert trimmed == want_trimmed, (ops, match)
            if want_score is not None:
                assert (c.score, c.end_v, c.end_h) == (want_score, ev, eh)
            # affine2p with the second model never cheaper is the affine rule
            # on runs
            cg2 = L.cigar_new(64)
            C.memmove(cg2.contents.operations, ops.encode(), len(ops))
            cg2.contents.begin_offset, cg2.contents.end_offset = 0, len(ops)
            a2 = wfa.Affine2pPenalties(match, 4, 6, 2, 1000, 1000)
            L.cigar_maxtrim_gap_affine2p(cg2, C.byref(a2))
            c2 = cg2.contents
            got2 = bytes(c2.operations[c2.begin_offset:c2.end_offset]).decode()
            assert len(got2) <= len(ops) and ops.startswith(got2)
            L.cigar_free(cg)
            L.cigar_free(cg2)
    # display
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    attr = wfa.default_attributes()
    h = L.wavefront_aligner_new(C.byref(attr))
    out = tmp_path / "conf.txt"
    fp = libc.fopen(str(out).encode(), b"w")
    for name in ("mode", "scope", "conf"):
        fn = getattr(L, f"wavefront_aligner_print_{name}")
        fn.argtypes = [C.c_void_p, C.c_void_p]
        fn(fp, h)
    libc.fclose(fp)
    assert out.read_text() == "WFA(alignment,end2end)(MHigh,inf)"
    L.wavefront_aligner_delete(h)


def test_fast_pass_kernel_table(wfa):
    """The two-diagonal fast pass's kernel table (wfa2-lib_gb300/csrc/wfa_fast2.cu):
    every (full CIGAR, o+e even, row width, default penalties, cut-off)
    instance the engine asks for exists, except the score-only cut-off kernel
    with rows of 1536 diagonals, which is not built (that second pass takes
    rows of 2048).  The table only hands out kernel addresses: no GPU call."""
    fn = wfa.lib().wf2g_fast2_kernel_ptr
    fn.restype = C.c_void_p
    fn.argtypes = [C.c_int] * 5
    for width in (1024, 1536, 2048):
        for cigar in (0, 1):
            assert fn(cigar, 1, width, 1, 0) and fn(cigar, 1, width, 0, 0), (width, cigar)
            assert fn(cigar, 0, width, 0, 0), (width, cigar)
            assert bool(fn(cigar, 1, width, 1, 1)) == (cigar == 1 or width != 1536), (width, cigar)
            assert not fn(cigar, 1, width, 0, 1), (width, cigar)  # cut-off: default penalties only
    assert not fn(1, 1, 512, 1, 0) and not fn(0, 1, 4096, 1, 0)

"""ctypes front-end for the CPU checker.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py.  Two back-ends share one
calling convention:

* ``port``      -- oracle/_build/libwfa_oracle.so, the C restatement of the
                   reference algorithm (wfa_oracle.c); builds on any host.
* ``reference`` -- oracle/_ref/libwfa_ref.so, the unmodified reference library
                   compiled from its sources (only where they are present).
* ``reference_scalar`` -- the same built without host tuning, so its portable
                   extension kernels run (the aarch64 behaviour; the x86 AVX
                   kernels resolve ends-free termination ties differently).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libwfa_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libwfa_ref.so")
REF_SCALAR_LIB = os.path.join(HERE, "_ref", "libwfa_ref_scalar.so")

INDEL, EDIT, GAP_LINEAR = 0, 1, 2
GAP_AFFINE = 3
GAP_AFFINE_2P = 4
MEM_HIGH, MEM_MED, MEM_LOW, MEM_ULTRALOW = 0, 1, 2, 3
FLAG_STALE_SOURCE, FLAG_OVER_BOUND = 1, 2


@dataclass
class Penalties:
    """Penalties as the reference's attribute structs hold them (match <= 0).
    Gap-linear keeps its indel penalty in gap_opening1; edit and indel take
    none."""

    metric: int = GAP_AFFINE
    match: int = 0
    mismatch: int = 4
    gap_opening1: int = 6
    gap_extension1: int = 2
    gap_opening2: int = 24
    gap_extension2: int = 1

    def cfg(self, memory_mode=MEM_HIGH, score_only=False, max_steps=0, wfadaptive=None,
            form=None, heuristic=None):
        """wfadaptive: None, or (min_wavefront_length, max_distance_threshold,
        steps_between_cutoffs) of the wf-adaptive heuristic.
        form: None (end-to-end), "extension", or the ends-free lengths
        (pattern_begin_free, pattern_end_free, text_begin_free, text_end_free).
        heuristic: None, or a Heuristic (any strategy set; overrides wfadaptive)."""
        h = [1, *wfadaptive] if wfadaptive else [0, 0, 0, 0]
        hx = [0, 0, 0, 0, 0]
        if heuristic is not None and heuristic.strategy:
            hz = heuristic
            h = [0, hz.min_wavefront_length, hz.max_distance_threshold, hz.steps_between_cutoffs]
            hx = [hz.strategy, hz.xdrop, hz.zdrop, hz.min_k, hz.max_k]
        if form is None:
            f = [0, 0, 0, 0, 0, 0]
        elif form == "extension":
            f = [1, 0, 0, 0, 0, 1]
        else:
            f = [1, *form, 0]
        return np.array(
            [self.metric, self.match, self.mismatch, self.gap_opening1, self.gap_extension1,
             self.gap_opening2, self.gap_extension2, memory_mode, int(bool(score_only)),
             max_steps, *h, *f, *hx], dtype=np.int32)


# wavefront/wavefront_heuristic.h:41-49
HS_BANDED_STATIC, HS_BANDED_ADAPTIVE, HS_WFADAPTIVE = 0x01, 0x02, 0x04
HS_XDROP, HS_ZDROP, HS_WFMASH = 0x10, 0x20, 0x40


@dataclass
class Heuristic:
    """A heuristic strategy (bit set of HS_*) and its parameters, as the
    reference's wavefront_heuristic_t holds them."""

    strategy: int = 0
    min_wavefront_length: int = 0
    max_distance_threshold: int = 0
    steps_between_cutoffs: int = 1
    xdrop: int = 0
    zdrop: int = 0
    min_k: int = 0
    max_k: int = 0


def build(ref: bool = False) -> None:
    targets = ["oracle"] + (["ref"] if ref else [])
    extra = [f"WFA_REF={os.environ['WFA_REF']}"] if os.environ.get("WFA_REF") else []
    subprocess.run(["make", "-s", "-C", HERE] + targets + extra, check=True)


_LIBS = {}


def _lib(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path = {"port": PORT_LIB, "reference": REF_LIB, "reference_scalar": REF_SCALAR_LIB}[kind]
    if not os.path.exists(path):
        build(ref=(kind != "port"))
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    if kind == "port":
        fn = lib.oracle_align_batch_flags
        fn.argtypes = [P, ctypes.c_int, P, P, P, P, P, P, P, P, P, P, P, P, P, P, ctypes.c_int]
    else:
        fn = lib.ref_align_batch
        fn.argtypes = [P, ctypes.c_int, P, P, P, P, P, P, P, P, P, P, P, P, P, ctypes.c_int]
    fn.restype = ctypes.c_int
    _LIBS[kind] = fn
    return fn


def reference_dir() -> str:
    """The reference's source tree: $WFA_REF, else the location this
    directory's Makefile builds the reference library from.  It exists only
    where the reference sources are present (not on the GPU hosts)."""
    env = os.environ.get("WFA_REF")
    if env:
        return env
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True,
                             text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""
    return out


def have_reference_sources() -> bool:
    d = reference_dir()
    return bool(d) and os.path.isdir(os.path.join(d, "wavefront"))


def have_reference() -> bool:
    return os.path.exists(REF_LIB)


@dataclass
class PairBatch:
    """Pairs packed as one ASCII buffer with offsets/lengths (the batch layout)."""

    seqs: np.ndarray  # uint8
    p_off: np.ndarray  # int64
    p_len: np.ndarray  # int32
    t_off: np.ndarray  # int64
    t_len: np.ndarray  # int32

    @property
    def n(self) -> int:
        return int(self.p_len.shape[0])

    @staticmethod
    def from_lists(patterns, texts) -> "PairBatch":
        parts, p_off, t_off = [], [], []
        pos = 0
        for p, t in zip(patterns, texts):
            pb = p.encode() if isinstance(p, str) else bytes(p)
            tb = t.encode() if isinstance(t, str) else bytes(t)
            p_off.append(pos)
            parts.append(pb)
            pos += len(pb)
            t_off.append(pos)
            parts.append(tb)
            pos += len(tb)
        buf = np.frombuffer(b"".join(parts) + b"\0" * 16, dtype=np.uint8).copy()
        return PairBatch(buf, np.array(p_off, np.int64),
                         np.array([len(p) for p in patterns], np.int32),
                         np.array(t_off, np.int64), np.array([len(t) for t in texts], np.int32))

    def pattern(self, i) -> bytes:
        o = int(self.p_off[i])
        return self.seqs[o:o + int(self.p_len[i])].tobytes()

    def text(self, i) -> bytes:
        o = int(self.t_off[i])
        return self.seqs[o:o + int(self.t_len[i])].tobytes()

    def ops_offsets(self) -> np.ndarray:
        cap = self.p_len.astype(np.int64) + self.t_len.astype(np.int64)
        off = np.zeros(self.n + 1, np.int64)
        np.cumsum(cap, out=off[1:])
        return off


@dataclass
class AlignResult:
    score: np.ndarray
    status: np.ndarray
    ops: np.ndarray  # uint8 buffer
    ops_off: np.ndarray  # int64 (n+1)
    ops_len: np.ndarray
    cells: np.ndarray
    ext: np.ndarray
    end: np.ndarray = None  # (n, 2) int32: cigar->end_v, cigar->end_h
    # ORACLE_FLAG_* bits (port only): FLAG_STALE_SOURCE marks a back-trace that
    # read a wavefront a heuristic cut had emptied
    flags: np.ndarray = None

    def cigar(self, i) -> str:
        if self.ops_len[i] < 0:
            return "<longer than plen+tlen>"
        o = int(self.ops_off[i])
        return self.ops[o:o + int(self.ops_len[i])].tobytes().decode()


def align(batch: PairBatch, pen: Penalties, memory_mode=MEM_HIGH, score_only=False,
          max_steps=0, kind="port", nthreads=0, wfadaptive=None, form=None,
          heuristic=None) -> AlignResult:
    fn = _lib(kind)
    n = batch.n
    cfg = pen.cfg(memory_mode, score_only, max_steps, wfadaptive, form, heuristic)
    score = np.zeros(n, np.int32)
    status = np.zeros(n, np.int32)
    ops_off = batch.ops_offsets()
    ops = np.zeros(max(int(ops_off[-1]), 1), np.uint8)
    ops_len = np.zeros(n, np.int32)
    cells = np.zeros(n, np.int64)
    ext = np.zeros(n, np.int64)
    end = np.zeros((n, 2), np.int32)

    def ptr(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    flags = np.zeros(n, np.int32)
    args = [ptr(cfg), n, ptr(batch.seqs), ptr(batch.p_off), ptr(batch.p_len), ptr(batch.t_off),
            ptr(batch.t_len), ptr(score), ptr(status), ptr(ops), ptr(ops_off), ptr(ops_len),
            ptr(cells), ptr(ext), ptr(end)]
    if kind == "port":
        args.append(ptr(flags))
    rc = fn(*args, int(nthreads))
    if rc != 0:
        raise ValueError("invalid configuration for the CPU checker")
    return AlignResult(score, status, ops, ops_off, ops_len, cells, ext, end, flags)


def compare(batch: PairBatch, pen: Penalties, scores, status, ops, ops_off, ops_len,
            ref: "AlignResult", score_only=False, nthreads=0) -> dict:
    """Pair-by-pair comparison of results under test (scores, status and, in
    full-CIGAR runs, ops/ops_off/ops_len) with the checker's `ref`, replaying
    and rescoring every CIGAR under test (oracle/wfa_check.c).  Returns the
    mismatch counts and the first differing pair (-1: none)."""
    lib = ctypes.CDLL(PORT_LIB) if os.path.exists(PORT_LIB) else None
    if lib is None:
        build()
        lib = ctypes.CDLL(PORT_LIB)
    fn = lib.oracle_compare_batch
    P = ctypes.c_void_p
    fn.argtypes = [P, ctypes.c_int] + [P] * 15 + [ctypes.c_int, P]
    fn.restype = ctypes.c_int
    cfg = pen.cfg(score_only=score_only)
    out = np.zeros(6, np.int64)

    def ptr(a):
        return None if a is None else np.ascontiguousarray(a).ctypes.data_as(P)
    keep = [np.ascontiguousarray(x) for x in (scores, status)]
    full = not score_only
    a_ops = np.ascontiguousarray(ops) if full else None
    a_off = np.ascontiguousarray(ops_off, dtype=np.int64) if full else None
    a_len = np.ascontiguousarray(ops_len, dtype=np.int32) if full else None
    fn(ptr(cfg), batch.n, ptr(batch.seqs), ptr(batch.p_off), ptr(batch.p_len), ptr(batch.t_off),
       ptr(batch.t_len), ptr(keep[0]), ptr(keep[1]), ptr(a_ops), ptr(a_off), ptr(a_len),
       ptr(ref.score), ptr(ref.status), ptr(ref.ops) if full else None,
       ptr(ref.ops_off) if full else None, ptr(ref.ops_len) if full else None, int(nthreads),
       ptr(out))
    return {"pairs_checked": int(batch.n), "score_mismatch": int(out[0]),
            "status_mismatch": int(out[1]), "cigar_mismatch": int(out[2]),
            "cigar_invalid": int(out[3]), "rescore_mismatch": int(out[4]),
            "first_bad_pair": int(out[5])}


# ---------------------------------------------------------------- formats
def read_seq_file(path) -> PairBatch:
    """Reads the reference's '.seq' format: '>pattern' / '<text' line pairs."""
    pats, txts = [], []
    with open(path, "rb") as f:
        lines = [l.rstrip(b"\r\n") for l in f if l.strip()]
    for i in range(0, len(lines) - 1, 2):
        assert lines[i][:1] == b">" and lines[i + 1][:1] == b"<"
        pats.append(lines[i][1:])
        txts.append(lines[i + 1][1:])
    return PairBatch.from_lists(pats, txts)


def cigar_rle(ops: str) -> str:
    """RLE as the reference prints it with matches shown (alignment/cigar.c:436-470)."""
    if not ops:
        return "-"
    out = []
    last, n = ops[0], 1
    for c in ops[1:]:
        if c == last:
            n += 1
        else:
            out.append(f"{n}{last}")
            last, n = c, 1
    out.append(f"{n}{last}")
    return "".join(out)


def rescore_affine(ops: str, match: int, x: int, o: int, e: int) -> int:
    """Score of a CIGAR under gap-affine penalties (alignment/cigar.c:277-303)."""
    score, last = 0, ""
    for c in ops:
        if c == "M":
            score -= match
        elif c == "X":
            score -= x
        elif c in "DI":
            score -= e + (0 if last == c else o)
        last = c
    return score


def rescore_affine2p(ops: str, match: int, x: int, o1: int, e1: int, o2: int, e2: int) -> int:
    """Score under gap-affine-2p penalties (alignment/cigar.c:304-346)."""
    def op_score(c, n):
        if c == "M":
            return match * n
        if c == "X":
            return x * n
        return min(o1 + e1 * n, o2 + e2 * n)
    if not ops:
        return 0
    score, last, n = 0, ops[0], 0
    for c in ops:
        if c != last:
            score -= op_score(last, n)
            last, n = c, 0
        n += 1
    score -= op_score(last, n)
    return score


def rescore(ops: str, pen: Penalties) -> int:
    """Score of a CIGAR under the metric (alignment/cigar.c:244-346): the edit
    or indel distance, or the negated gap-linear / affine / affine-2p cost
    (gap-linear takes its indel penalty from gap_opening1)."""
    if pen.metric in (INDEL, EDIT):
        return sum(1 for c in ops if c in "XID")
    if pen.metric == GAP_LINEAR:
        return -sum(pen.match if c == "M" else pen.mismatch if c == "X" else pen.gap_opening1
                    for c in ops)
    if pen.metric == GAP_AFFINE:
        return rescore_affine(ops, pen.match, pen.mismatch, pen.gap_opening1, pen.gap_extension1)
    return rescore_affine2p(ops, pen.match, pen.mismatch, pen.gap_opening1, pen.gap_extension1,
                            pen.gap_opening2, pen.gap_extension2)


def check_cigar(ops: str, pattern: bytes, text: bytes) -> bool:
    """Replays a CIGAR against its sequences (alignment/cigar.c:347-420)."""
    v = h = 0
    for c in ops:
        if c == "M":
            if v >= len(pattern) or h >= len(text) or pattern[v] != text[h]:
                return False
            v += 1
            h += 1
        elif c == "X":
            if v >= len(pattern) or h >= len(text) or pattern[v] == text[h]:
                return False
            v += 1
            h += 1
        elif c == "I":
            h += 1
        elif c == "D":
            v += 1
        else:
            return False
    return v == len(pattern) and h == len(text)

"""Python host mirror of the GB300 wavefront aligner's C ABI (include/wfa2gpu.h).

The product is the C library lib/libwfa2gpu.so; this module binds it with
ctypes so tests and benchmarks can drive the same entry points a C caller of
WFA2-lib uses (``wavefront_aligner_new`` / ``wavefront_align`` / ``cigar_t``)
plus the batch calls.  It never computes an alignment itself: if the library
or a GPU is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time
from dataclasses import dataclass

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libwfa2gpu.so")
GEN_PATH = os.path.join(PKG_DIR, "lib", "libwfa2gen.so")

# wavefront/wfa.h:46-55
WF_STATUS_ALG_COMPLETED = 0
WF_STATUS_ALG_PARTIAL = 1
WF_STATUS_MAX_STEPS_REACHED = -100
WF_STATUS_OOM = -200
WF_STATUS_UNATTAINABLE = -300
WF2G_STATUS_INVALID_FORM = -400  # ends-free lengths longer than a pair's sequences
ALIGNMENT_END2END, ALIGNMENT_ENDSFREE = 0, 1

INDEL, EDIT, GAP_LINEAR, GAP_AFFINE, GAP_AFFINE_2P = 0, 1, 2, 3, 4
COMPUTE_SCORE, COMPUTE_ALIGNMENT = 0, 1
MEM_HIGH, MEM_MED, MEM_LOW, MEM_ULTRALOW = 0, 1, 2, 3
WF_HEURISTIC_NONE = 0
# wavefront/wavefront_heuristic.h:41-49
WF_HEURISTIC_BANDED_STATIC = 0x1
WF_HEURISTIC_BANDED_ADAPTIVE = 0x2
WF_HEURISTIC_WFADAPTIVE = 0x4
WF_HEURISTIC_XDROP = 0x10
WF_HEURISTIC_ZDROP = 0x20
WF_HEURISTIC_WFMASH = 0x40


# ------------------------------------------------------------ ABI mirror
class LinearPenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("indel", C.c_int)]


class AffinePenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("gap_opening", C.c_int),
                ("gap_extension", C.c_int)]


class Affine2pPenalties(C.Structure):
    _fields_ = [("match", C.c_int), ("mismatch", C.c_int), ("gap_opening1", C.c_int),
                ("gap_extension1", C.c_int), ("gap_opening2", C.c_int),
                ("gap_extension2", C.c_int)]


class AlignmentForm(C.Structure):
    _fields_ = [("span", C.c_int), ("extension", C.c_bool), ("pattern_begin_free", C.c_int),
                ("pattern_end_free", C.c_int), ("text_begin_free", C.c_int),
                ("text_end_free", C.c_int)]


class ProfilerCounter(C.Structure):
    _fields_ = [("total", C.c_uint64), ("samples", C.c_uint64), ("min", C.c_uint64),
                ("max", C.c_uint64), ("m_oldM", C.c_double), ("m_newM", C.c_double),
                ("m_oldS", C.c_double), ("m_newS", C.c_double)]


class Timespec(C.Structure):
    _fields_ = [("tv_sec", C.c_long), ("tv_nsec", C.c_long)]


class ProfilerTimer(C.Structure):
    _fields_ = [("begin_timer", Timespec), ("time_ns", ProfilerCounter),
                ("accumulated", C.c_uint64)]


class AlignmentSystem(C.Structure):
    _fields_ = [("max_alignment_steps", C.c_int), ("probe_interval_global", C.c_int),
                ("probe_interval_compact", C.c_int), ("max_partial_compacts", C.c_uint64),
                ("max_memory_compact", C.c_uint64), ("max_memory_resident", C.c_uint64),
                ("max_memory_abort", C.c_uint64), ("verbose", C.c_int),
                ("check_alignment_correct", C.c_bool), ("timer", ProfilerTimer),
                ("max_num_threads", C.c_int), ("min_offsets_per_thread", C.c_int)]


class Heuristic(C.Structure):
    _fields_ = [("strategy", C.c_uint), ("steps_between_cutoffs", C.c_int), ("min_k", C.c_int),
                ("max_k", C.c_int), ("min_wavefront_length", C.c_int),
                ("max_distance_threshold", C.c_int), ("xdrop", C.c_int), ("zdrop", C.c_int),
                ("steps_wait", C.c_int), ("max_sw_score", C.c_int), ("max_wf_score", C.c_int),
                ("max_sw_score_offset", C.c_int), ("max_sw_score_k", C.c_int)]


class PlotAttr(C.Structure):
    _fields_ = [("enabled", C.c_bool), ("resolution_points", C.c_int), ("align_level", C.c_int)]


class AlignerAttr(C.Structure):
    _fields_ = [("distance_metric", C.c_int), ("alignment_scope", C.c_int),
                ("alignment_form", AlignmentForm), ("linear_penalties", LinearPenalties),
                ("affine_penalties", AffinePenalties), ("affine2p_penalties", Affine2pPenalties),
                ("heuristic", Heuristic), ("memory_mode", C.c_int),
                ("mm_allocator", C.c_void_p), ("plot", PlotAttr), ("system", AlignmentSystem)]


class Cigar(C.Structure):
    _fields_ = [("operations", C.POINTER(C.c_char)), ("max_operations", C.c_int),
                ("begin_offset", C.c_int), ("end_offset", C.c_int), ("score", C.c_int),
                ("end_v", C.c_int), ("end_h", C.c_int), ("has_misms", C.c_bool),
                ("cigar_buffer", C.POINTER(C.c_uint32)), ("cigar_length", C.c_int)]


class AlignStatus(C.Structure):
    _fields_ = [("status", C.c_int), ("score", C.c_int), ("dropped", C.c_bool),
                ("num_null_steps", C.c_int), ("memory_used", C.c_uint64),
                ("wf_align_compute", C.c_void_p), ("wf_align_extend", C.c_void_p)]


class WavefrontPenalties(C.Structure):
    _fields_ = [("distance_metric", C.c_int), ("match", C.c_int), ("mismatch", C.c_int),
                ("gap_opening1", C.c_int), ("gap_extension1", C.c_int),
                ("gap_opening2", C.c_int), ("gap_extension2", C.c_int),
                ("linear_penalties", LinearPenalties), ("affine_penalties", AffinePenalties),
                ("affine2p_penalties", Affine2pPenalties), ("internal_gap_e", C.c_int)]


class Aligner_t(C.Structure):
    _fields_ = [("align_mode", C.c_int), ("align_mode_tag", C.c_char_p),
                ("align_status", AlignStatus), ("alignment_scope", C.c_int),
                ("alignment_form", AlignmentForm), ("penalties", WavefrontPenalties),
                ("heuristic", Heuristic), ("memory_mode", C.c_int),
                ("cigar", C.POINTER(Cigar)), ("system", AlignmentSystem),
                ("bialigner", C.c_void_p), ("engine", C.c_void_p)]


# exported symbols of include/wfa2gpu.h (checked by the CPU test-suite)
EXPORTED = [
    "wavefront_aligner_attr_default", "wavefront_align_strerror",
    "wavefront_align_strerror_short", "wavefront_aligner_new", "wavefront_aligner_reap",
    "wavefront_aligner_delete", "wavefront_aligner_set_alignment_end_to_end",
    "wavefront_aligner_set_alignment_free_ends", "wavefront_aligner_set_alignment_extension",
    "wavefront_aligner_set_heuristic_none", "wavefront_aligner_set_heuristic_wfadaptive",
    "wavefront_aligner_set_heuristic_wfmash", "wavefront_aligner_set_heuristic_xdrop",
    "wavefront_aligner_set_heuristic_zdrop", "wavefront_aligner_set_heuristic_banded_static",
    "wavefront_aligner_set_heuristic_banded_adaptive",
    "wavefront_aligner_set_max_alignment_steps", "wavefront_aligner_set_max_memory",
    "wavefront_aligner_set_max_num_threads", "wavefront_aligner_set_min_offsets_per_thread",
    "wavefront_align", "wavefront_align_lambda", "wavefront_align_packed2bits",
    "cigar_new", "cigar_clear", "cigar_resize", "cigar_free", "cigar_is_null",
    "cigar_count_matches", "cigar_get_CIGAR", "cigar_score_edit", "cigar_score_gap_linear",
    "cigar_score_gap_affine", "cigar_score_gap_affine2p", "cigar_check_alignment",
    "cigar_print", "cigar_sprint", "cigar_print_SAM_CIGAR", "cigar_sprint_SAM_CIGAR",
    "cigar_print_pretty", "wavefront_align_batch", "wavefront_align_batch_ends",
    "wavefront_align_batch_device",
    "wavefront_aligner_gpu_launches", "wfa2gpu_device",
    "wavefront_align_batch_device_noalloc",
    "wavefront_server_new", "wavefront_server_submit", "wavefront_server_poll",
    "wavefront_server_in_flight", "wavefront_server_gpu_launches", "wavefront_server_delete",
]


class ServerAttr(C.Structure):
    """wavefront_server_attr_t"""
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("backtrace_budget_bytes", C.c_int64),
                ("lanes", C.c_int),
                ("max_batch_pairs", C.c_int), ("batch_window_us", C.c_int),
                ("biwfa_min_length", C.c_int)]


class ServerResult(C.Structure):
    """wavefront_server_result_t"""
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("score", C.c_int),
                ("memory_mode", C.c_int), ("operations", C.c_void_p),
                ("operations_length", C.c_int), ("latency_us", C.c_double)]


def build() -> None:
    """Compiles lib/libwfa2gpu.so and lib/libwfa2gen.so in-tree (nvcc, sm_103a)."""
    subprocess.run(["make", "-s", "-C", PKG_DIR, f"-j{min(8, os.cpu_count() or 1)}"], check=True)


_lib = None


def lib() -> C.CDLL:
    """Loads libwfa2gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    L.wavefront_aligner_new.argtypes = [C.POINTER(AlignerAttr)]
    L.wavefront_aligner_new.restype = C.POINTER(Aligner_t)
    L.wavefront_aligner_delete.argtypes = [C.POINTER(Aligner_t)]
    L.wavefront_aligner_delete.restype = None
    L.wavefront_align.argtypes = [C.POINTER(Aligner_t), C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    L.wavefront_align.restype = C.c_int
    L.wavefront_align_packed2bits.argtypes = [C.POINTER(Aligner_t), P, C.c_int, P, C.c_int]
    L.wavefront_align_packed2bits.restype = C.c_int
    L.wavefront_align_batch.argtypes = [C.POINTER(Aligner_t), C.c_int, P, P, P, P, P, P, P, P,
                                        P, P]
    L.wavefront_align_batch.restype = C.c_int
    L.wavefront_align_batch_ends.argtypes = [C.POINTER(Aligner_t), C.c_int, P, P, P, P, P, P, P,
                                             P, P, P, P]
    L.wavefront_align_batch_ends.restype = C.c_int
    L.wavefront_align_batch_device.argtypes = [C.POINTER(Aligner_t), C.c_int, P, P, P, P, P,
                                               C.c_int, P, P, P, P, P, P]
    L.wavefront_align_batch_device.restype = C.c_int
    L.wavefront_align_batch_device_noalloc.argtypes = [C.POINTER(Aligner_t), C.c_int, P, P, P,
                                                       P, P, C.c_int, P, P, P, P, P, P]
    L.wavefront_align_batch_device_noalloc.restype = C.c_int
    L.wavefront_aligner_gpu_launches.argtypes = [C.POINTER(Aligner_t)]
    L.wavefront_aligner_gpu_launches.restype = C.c_int64
    L.wfa2gpu_device.restype = C.c_int
    L.wavefront_align_strerror.argtypes = [C.c_int]
    L.wavefront_align_strerror.restype = C.c_char_p
    L.cigar_sprint.argtypes = [C.c_char_p, C.POINTER(Cigar), C.c_bool]
    L.cigar_sprint.restype = C.c_int
    L.cigar_score_gap_affine.argtypes = [C.POINTER(Cigar), C.POINTER(AffinePenalties)]
    L.cigar_score_gap_affine.restype = C.c_int
    L.cigar_score_gap_affine2p.argtypes = [C.POINTER(Cigar), C.POINTER(Affine2pPenalties)]
    L.cigar_score_gap_affine2p.restype = C.c_int
    L.cigar_check_alignment.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int,
                                        C.POINTER(Cigar), C.c_bool]
    L.cigar_check_alignment.restype = C.c_bool
    L.wavefront_server_new.argtypes = [C.POINTER(Aligner_t), C.POINTER(ServerAttr)]
    L.wavefront_server_new.restype = C.c_void_p
    L.wavefront_server_submit.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    L.wavefront_server_submit.restype = C.c_int64
    L.wavefront_server_poll.argtypes = [C.c_void_p, C.POINTER(ServerResult), C.c_int, C.c_int]
    L.wavefront_server_poll.restype = C.c_int
    L.wavefront_server_in_flight.argtypes = [C.c_void_p]
    L.wavefront_server_in_flight.restype = C.c_int64
    L.wavefront_server_gpu_launches.argtypes = [C.c_void_p]
    L.wavefront_server_gpu_launches.restype = C.c_int64
    L.wavefront_server_delete.argtypes = [C.c_void_p]
    L.wavefront_server_delete.restype = None
    _lib = L
    return L


def default_attributes() -> AlignerAttr:
    """A copy of the exported ``wavefront_aligner_attr_default`` global."""
    a = AlignerAttr.in_dll(lib(), "wavefront_aligner_attr_default")
    c = AlignerAttr()
    C.memmove(C.byref(c), C.byref(a), C.sizeof(AlignerAttr))
    return c


@dataclass
class Config:
    """What the reference's attribute object configures for this path."""

    metric: int = GAP_AFFINE
    match: int = 0
    mismatch: int = 4
    gap_opening1: int = 6
    gap_extension1: int = 2
    gap_opening2: int = 24
    gap_extension2: int = 1
    score_only: bool = False
    memory_mode: int = MEM_HIGH
    max_steps: int = 0
    # wf-adaptive heuristic: (min_wavefront_length, max_distance_threshold,
    # steps_between_cutoffs), or None for exact alignment
    wfadaptive: tuple | None = None
    # alignment form: None (end-to-end), "extension", or the ends-free lengths
    # (pattern_begin_free, pattern_end_free, text_begin_free, text_end_free)
    form: tuple | str | None = None
    # any heuristic strategy set (overrides wfadaptive): a dict with
    # "strategy" (WF_HEURISTIC_* bits) and the wavefront_heuristic_t fields it
    # uses (min_wavefront_length, max_distance_threshold,
    # steps_between_cutoffs, xdrop, zdrop, min_k, max_k)
    heuristic: dict | None = None

    def attributes(self) -> AlignerAttr:
        a = default_attributes()
        a.distance_metric = self.metric
        a.alignment_scope = COMPUTE_SCORE if self.score_only else COMPUTE_ALIGNMENT
        a.affine_penalties.match = self.match
        a.affine_penalties.mismatch = self.mismatch
        a.affine_penalties.gap_opening = self.gap_opening1
        a.affine_penalties.gap_extension = self.gap_extension1
        a.affine2p_penalties.match = self.match
        a.affine2p_penalties.mismatch = self.mismatch
        a.affine2p_penalties.gap_opening1 = self.gap_opening1
        a.affine2p_penalties.gap_extension1 = self.gap_extension1
        a.affine2p_penalties.gap_opening2 = self.gap_opening2
        a.affine2p_penalties.gap_extension2 = self.gap_extension2
        # gap-linear: the indel penalty is gap_opening1 (edit and indel take none)
        a.linear_penalties.match = self.match
        a.linear_penalties.mismatch = self.mismatch
        a.linear_penalties.indel = self.gap_opening1
        a.heuristic.strategy = WF_HEURISTIC_NONE
        if self.wfadaptive:
            a.heuristic.strategy = WF_HEURISTIC_WFADAPTIVE
            (a.heuristic.min_wavefront_length, a.heuristic.max_distance_threshold,
             a.heuristic.steps_between_cutoffs) = self.wfadaptive
        if self.heuristic:
            for key, value in self.heuristic.items():
                setattr(a.heuristic, key, value)
        a.memory_mode = self.memory_mode
        if self.max_steps > 0:
            a.system.max_alignment_steps = self.max_steps
        f = a.alignment_form
        f.span, f.extension = ALIGNMENT_END2END, False
        f.pattern_begin_free = f.pattern_end_free = f.text_begin_free = f.text_end_free = 0
        if self.form == "extension":
            f.span, f.extension = ALIGNMENT_ENDSFREE, True
        elif self.form is not None:
            f.span = ALIGNMENT_ENDSFREE
            (f.pattern_begin_free, f.pattern_end_free, f.text_begin_free,
             f.text_end_free) = self.form
        return a


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


class Aligner:
    """One ``wavefront_aligner_t`` (one GPU engine and stream)."""

    def __init__(self, cfg: Config | None = None):
        self.cfg = cfg or Config()
        self._attr = self.cfg.attributes()
        self._h = lib().wavefront_aligner_new(C.byref(self._attr))
        if not self._h:
            raise RuntimeError("wavefront_aligner_new failed")
        if not self._h.contents.engine:
            raise RuntimeError("no usable GPU: the GB300 aligner has no CPU fallback")

    def close(self):
        if getattr(self, "_h", None):
            lib().wavefront_aligner_delete(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def launches(self) -> int:
        return int(lib().wavefront_aligner_gpu_launches(self._h))

    # -------------------------------------------------- per pair (drop-in)
    def align(self, pattern: bytes, text: bytes):
        """wavefront_align(); returns (status, cigar->score, operations)."""
        st = lib().wavefront_align(self._h, pattern, len(pattern), text, len(text))
        cg = self._h.contents.cigar.contents
        ops = b""
        if cg.end_offset > cg.begin_offset:
            ops = C.string_at(C.addressof(cg.operations.contents) + cg.begin_offset,
                              cg.end_offset - cg.begin_offset)
        return st, cg.score, ops.decode()

    def align_packed2bits(self, pattern: bytes, plen: int, text: bytes, tlen: int):
        pa = np.frombuffer(pattern, np.uint8)
        ta = np.frombuffer(text, np.uint8)
        st = lib().wavefront_align_packed2bits(self._h, _ptr(pa), plen, _ptr(ta), tlen)
        cg = self._h.contents.cigar.contents
        ops = b""
        if cg.end_offset > cg.begin_offset:
            ops = C.string_at(C.addressof(cg.operations.contents) + cg.begin_offset,
                              cg.end_offset - cg.begin_offset)
        return st, cg.score, ops.decode()

    # ---------------------------------------------------------------- batch
    def align_batch(self, seqs, p_off, p_len, t_off, t_len, ops_off=None, scores=None,
                    status=None, ops=None, ops_len=None):
        """wavefront_align_batch() on host arrays; returns (rc, scores, status, ops, ops_len)."""
        n = int(p_len.shape[0])
        scores = np.zeros(n, np.int32) if scores is None else scores
        status = np.zeros(n, np.int32) if status is None else status
        if not self.cfg.score_only:
            if ops_off is None:
                ops_off = np.zeros(n + 1, np.int64)
                np.cumsum(p_len.astype(np.int64) + t_len.astype(np.int64), out=ops_off[1:])
            if ops is None:
                ops = np.zeros(max(int(ops_off[n] if ops_off.shape[0] > n else
                                       ops_off[-1] + p_len[-1] + t_len[-1]), 1), np.uint8)
            if ops_len is None:
                ops_len = np.zeros(n, np.int32)
        rc = lib().wavefront_align_batch(self._h, n, _ptr(seqs), _ptr(p_off), _ptr(p_len),
                                         _ptr(t_off), _ptr(t_len), _ptr(scores), _ptr(status),
                                         _ptr(ops), _ptr(ops_off), _ptr(ops_len))
        return rc, scores, status, ops, ops_len, ops_off

    def align_batch_ends(self, seqs, p_off, p_len, t_off, t_len):
        """wavefront_align_batch_ends(); returns (rc, scores, status, ops, ops_len, ops_off,
        end_info) with end_info an (n, 3) array of cigar->end_v, cigar->end_h and the WFA
        score."""
        n = int(p_len.shape[0])
        scores = np.zeros(n, np.int32)
        status = np.zeros(n, np.int32)
        end_info = np.zeros((n, 3), np.int32)
        ops = ops_off = ops_len = None
        if not self.cfg.score_only:
            ops_off = np.zeros(n + 1, np.int64)
            np.cumsum(p_len.astype(np.int64) + t_len.astype(np.int64), out=ops_off[1:])
            ops = np.zeros(max(int(ops_off[n]), 1), np.uint8)
            ops_len = np.zeros(n, np.int32)
        rc = lib().wavefront_align_batch_ends(self._h, n, _ptr(seqs), _ptr(p_off), _ptr(p_len),
                                              _ptr(t_off), _ptr(t_len), _ptr(scores),
                                              _ptr(status), _ptr(ops), _ptr(ops_off),
                                              _ptr(ops_len), _ptr(end_info))
        return rc, scores, status, ops, ops_len, ops_off, end_info

    def align_batch_device(self, n, d_seqs, d_poff, d_plen, d_toff, d_tlen, max_len, d_scores,
                           d_status, d_ops=0, d_ops_off=0, d_ops_len=0, stream=0) -> int:
        """wavefront_align_batch_device() with raw device pointers (ints)."""
        V = C.c_void_p
        return lib().wavefront_align_batch_device(
            self._h, n, V(d_seqs), V(d_poff), V(d_plen), V(d_toff), V(d_tlen), int(max_len),
            V(d_scores), V(d_status), V(d_ops), V(d_ops_off), V(d_ops_len), V(stream))


    def align_batch_device_noalloc(self, n, d_seqs, d_poff, d_plen, d_toff, d_tlen, max_len,
                                   d_scores, d_status, d_ops=0, d_ops_off=0, d_ops_len=0,
                                   stream=0) -> int:
        """wavefront_align_batch_device_noalloc(): same arguments, no allocation."""
        V = C.c_void_p
        return lib().wavefront_align_batch_device_noalloc(
            self._h, n, V(d_seqs), V(d_poff), V(d_plen), V(d_toff), V(d_tlen), int(max_len),
            V(d_scores), V(d_status), V(d_ops), V(d_ops_off), V(d_ops_len), V(stream))


# ------------------------------------------------------------ generator
_gen = None


def _genlib():
    global _gen
    if _gen is None:
        if not os.path.exists(GEN_PATH):
            raise RuntimeError(f"{GEN_PATH} is missing: build the library first")
        g = C.CDLL(GEN_PATH)
        g.wf2g_generate_lengths.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int,
                                            C.c_void_p, C.c_void_p]
        g.wf2g_generate_pairs.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_void_p]
        _gen = g
    return _gen


class Server:
    """A ``wavefront_server_t``: continuous batching of single-pair requests."""

    def __init__(self, cfg: Config | None = None, hbm_budget_bytes: int = 0, lanes: int = 0,
                 max_batch_pairs: int = 0, batch_window_us: int = -1,
                 backtrace_budget_bytes: int = 0, biwfa_min_length: int = 0):
        self.cfg = cfg or Config()
        self._al = Aligner(self.cfg)
        attr = ServerAttr(hbm_budget_bytes, backtrace_budget_bytes, lanes, max_batch_pairs,
                          batch_window_us, biwfa_min_length)
        self._h = lib().wavefront_server_new(self._al._h, C.byref(attr))
        if not self._h:
            raise RuntimeError("wavefront_server_new failed")
        self._res = (ServerResult * 4096)()

    def submit(self, pattern: bytes, text: bytes) -> int:
        rid = int(lib().wavefront_server_submit(self._h, pattern, len(pattern), text, len(text)))
        if rid < 0:
            raise RuntimeError(f"wavefront_server_submit failed: {rid}")
        return rid

    def poll(self, timeout_us: int = 1000):
        """Finished results: list of (id, status, score, memory_mode, ops, latency_us)."""
        k = lib().wavefront_server_poll(self._h, self._res, len(self._res), timeout_us)
        out = []
        for r in self._res[:max(k, 0)]:
            ops = C.string_at(r.operations, r.operations_length).decode() if r.operations_length else ""
            out.append((r.id, r.status, r.score, r.memory_mode, ops, r.latency_us))
        return out

    def wait_all(self, ids, timeout_s: float = 600.0):
        """Polls until every id in `ids` has returned; {id: result tuple}."""
        want = set(ids)
        got = {}
        t0 = time.time()
        while want - got.keys():
            for r in self.poll(10_000):
                got[r[0]] = r
            if time.time() - t0 > timeout_s:
                raise TimeoutError(f"{len(want - got.keys())} requests still in flight")
        return got

    @property
    def in_flight(self) -> int:
        return int(lib().wavefront_server_in_flight(self._h))

    @property
    def launches(self) -> int:
        return int(lib().wavefront_server_gpu_launches(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().wavefront_server_delete(self._h)
            self._h = None
        if getattr(self, "_al", None):
            self._al.close()
            self._al = None

    def __del__(self):
        self.close()


@dataclass
class Pairs:
    seqs: np.ndarray
    p_off: np.ndarray
    p_len: np.ndarray
    t_off: np.ndarray
    t_len: np.ndarray

    @property
    def n(self):
        return int(self.p_len.shape[0])

    @property
    def max_len(self):
        return int(max(self.p_len.max(initial=0), self.t_len.max(initial=0)))

    def pattern(self, i) -> bytes:
        o = int(self.p_off[i])
        return self.seqs[o:o + int(self.p_len[i])].tobytes()

    def text(self, i) -> bytes:
        o = int(self.t_off[i])
        return self.seqs[o:o + int(self.t_len[i])].tobytes()


def generate(workload: int, n: int, first: int = 0, param: int = 0, param2: int = 0,
             alloc=None) -> Pairs:
    """Seeded synthetic pairs [first, first+n) of a workload (see wfa_datagen.c).

    ``alloc(nbytes) -> np.ndarray[uint8]`` may supply the sequence buffer
    (e.g. pinned host memory)."""
    g = _genlib()
    p_len = np.zeros(n, np.int32)
    t_len = np.zeros(n, np.int32)
    g.wf2g_generate_lengths(workload, first, n, param, param2, _ptr(p_len), _ptr(t_len))
    both = np.empty(2 * n, np.int64)
    both[0::2] = p_len
    both[1::2] = t_len
    ends = np.cumsum(both)
    starts = ends - both
    p_off = np.ascontiguousarray(starts[0::2])
    t_off = np.ascontiguousarray(starts[1::2])
    total = int(ends[-1]) if n else 0
    seqs = alloc(total + 16) if alloc else np.zeros(total + 16, np.uint8)
    g.wf2g_generate_pairs(workload, first, n, param, param2, _ptr(seqs), _ptr(p_off), _ptr(t_off))
    return Pairs(seqs, p_off, p_len, t_off, t_len)

"""Shared helpers of the test-suite: golden fixtures and result comparison."""
import gzip
import json
import os
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def crc(s: str) -> int:
    return zlib.crc32(s.encode()) & 0xFFFFFFFF


def utest_pairs():
    """The reference test-suite's 305 pairs as (patterns, texts) bytes lists."""
    with gzip.open(os.path.join(GOLDEN, "utest.seq.gz"), "rb") as f:
        lines = [l.rstrip(b"\r\n") for l in f.read().split(b"\n") if l.strip()]
    pats = [lines[i][1:] for i in range(0, len(lines), 2)]
    txts = [lines[i + 1][1:] for i in range(0, len(lines), 2)]
    return pats, txts


def utest_expected():
    with open(os.path.join(GOLDEN, "utest_expected.json")) as f:
        return json.load(f)


def synthetic_expected():
    with open(os.path.join(GOLDEN, "synthetic_expected.json")) as f:
        return json.load(f)


def endsfree_expected():
    """Reference outputs for the ends-free and extension forms; a fixture's
    "form" is a list of the four free lengths or the string "extension"."""
    with open(os.path.join(GOLDEN, "endsfree_expected.json")) as f:
        d = json.load(f)
    for fx in d.values():
        if isinstance(fx["form"], list):
            fx["form"] = tuple(fx["form"])
        if fx["wfadaptive"] is not None:
            fx["wfadaptive"] = tuple(fx["wfadaptive"])
    return d


def heuristics_expected():
    """Reference outputs under the heuristics other than wf-adaptive; a
    fixture's "keep" lists the generated pairs it holds rows for."""
    with open(os.path.join(GOLDEN, "heuristics_expected.json")) as f:
        d = json.load(f)
    for fx in d.values():
        if isinstance(fx["form"], list):
            fx["form"] = tuple(fx["form"])
    return d


def heuristic_pairs(O, W, fx):
    """The kept pairs of a heuristic fixture set, as one PairBatch."""
    p = W.generate(fx["workload"], fx["n"], param=fx["param"], param2=fx["param2"])
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    return O.PairBatch.from_lists([b.pattern(i) for i in fx["keep"]],
                                  [b.text(i) for i in fx["keep"]])


def pack(patterns, texts):
    """Concatenated ASCII batch: (seqs, p_off, p_len, t_off, t_len)."""
    parts, p_off, t_off, pos = [], [], [], 0
    for p, t in zip(patterns, texts):
        p_off.append(pos)
        parts.append(p)
        pos += len(p)
        t_off.append(pos)
        parts.append(t)
        pos += len(t)
    seqs = np.frombuffer(b"".join(parts) + b"\0" * 16, np.uint8).copy()
    return (seqs, np.array(p_off, np.int64), np.array([len(p) for p in patterns], np.int32),
            np.array(t_off, np.int64), np.array([len(t) for t in texts], np.int32))


def rle(ops: str) -> str:
    if not ops:
        return "-"
    out, last, n = [], ops[0], 0
    for c in ops:
        if c == last:
            n += 1
        else:
            out.append(f"{n}{last}")
            last, n = c, 1
    out.append(f"{n}{last}")
    return "".join(out)

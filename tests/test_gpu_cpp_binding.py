"""The C++ WFAligner classes on the GPU: a C++ program built against
include/bindings/cpp/WFAligner.hpp aligns pairs per call (end-to-end, ends-free,
extension) and in one alignBatch() call; every result equals the CPU
checker's, and getCIGAR() is the run-length SAM CIGAR of the operations
('=' match, 'X' mismatch; alignment/cigar.c:181-243)."""
import shutil

import pytest

import helpers
from test_cpp_binding import build_driver

pytestmark = pytest.mark.gpu

PENS = {
    "affine": dict(metric=3),
    "affine2p": dict(metric=4),
    "edit": dict(metric=1),
    "indel": dict(metric=0),
    "linear": dict(metric=2, match=0, mismatch=4, gap_opening1=2),
}


def _sam(ops):
    out, last, n = [], None, 0
    for c in ops:
        c = "=" if c == "M" else c
        if c != last and last is not None:
            out.append(f"{n}{last}")
            n = 0
        last = c
        n += 1
    if last is not None:
        out.append(f"{n}{last}")
    return "".join(out)


@pytest.fixture(scope="module")
def driver(tmp_path_factory, wfa):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("cpp") / "driver")
    build_driver(exe)
    return exe


@pytest.mark.parametrize("metric", sorted(PENS))
@pytest.mark.parametrize("form", ["e2e", "ext", "ef:0,20,0,20"])
def test_cpp_classes_match_oracle(gpu_available, wfa, oracle_mod, driver, metric, form):
    import subprocess
    W, O = wfa, oracle_mod
    p = W.generate(1, 40, first=2024)
    lines = "".join(f"{p.pattern(i).decode()}\t{p.text(i).decode()}\n" for i in range(p.n))
    r = subprocess.run([driver, metric, form], input=lines, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [l.split("\t") for l in r.stdout.splitlines()]
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    oform = None if form == "e2e" else "extension" if form == "ext" else (0, 20, 0, 20)
    want = O.align(b, O.Penalties(**PENS[metric]), form=oform)
    for i, (st, sc, ops, sam) in enumerate(rows):
        assert (int(st), int(sc), ops) == (int(want.status[i]), int(want.score[i]),
                                            want.cigar(i)), (metric, form, i)
        assert sam == _sam(ops), i


def test_cpp_batch_matches_oracle(gpu_available, wfa, oracle_mod, driver):
    import subprocess
    W, O = wfa, oracle_mod
    p = W.generate(1, 200, first=77)
    lines = "".join(f"{p.pattern(i).decode()}\t{p.text(i).decode()}\n" for i in range(p.n))
    r = subprocess.run([driver, "affine", "e2e", "batch"], input=lines, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    want = O.align(b, O.Penalties())
    for i, row in enumerate(r.stdout.splitlines()):
        st, sc, ops = row.split("\t")
        assert (int(st), int(sc), ops) == (int(want.status[i]), int(want.score[i]),
                                            want.cigar(i)), i

"""Seeded synthetic generator: determinism and workload shapes (CPU only)."""
import numpy as np


def test_deterministic_and_subrange(wfa):
    a = wfa.generate(1, 300)
    b = wfa.generate(1, 300)
    assert np.array_equal(a.seqs, b.seqs)
    c = wfa.generate(1, 100, first=200)
    for i in range(100):
        assert c.pattern(i) == a.pattern(200 + i) and c.text(i) == a.text(200 + i)


def test_workload_shapes(wfa):
    w0 = wfa.generate(0, 2000)
    assert (w0.p_len == 100).all() and abs(int(w0.t_len.sum()) - 200000) < 2000
    w1 = wfa.generate(1, 5000)
    assert w1.p_len.min() >= 500 and w1.p_len.max() <= 1500
    w2 = wfa.generate(2, 500)
    assert w2.p_len.min() >= 1000 and w2.p_len.max() <= 10000
    w4 = wfa.generate(4, 2000)
    assert w4.p_len.min() >= 100 and w4.p_len.max() <= 50000
    assert 1500 < np.median(w4.p_len) < 2600
    for p in (w0, w1):
        assert set(np.unique(p.seqs[:int(p.t_off[-1] + p.t_len[-1])]).tolist()) <= set(b"ACGT")


def test_pinned_checksum(wfa):
    """Bytes of the first pairs are pinned, so every host generates the same data."""
    import zlib
    p = wfa.generate(1, 50)
    assert zlib.crc32(p.seqs[:int(p.t_off[-1] + p.t_len[-1])].tobytes()) == PINNED_W1_50


PINNED_W1_50 = 2647829589

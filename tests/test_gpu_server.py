"""The serving loop (continuous batching) through the C ABI: every result is
the same alone and in a mix with other requests, equals the batch path in the
memory mode actually used (high, or ultralow for pairs re-run in BiWFA mode
after exceeding the back-trace budget), and matches the CPU checker.
Integer work: equality is exact."""
import threading

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

MEM_HIGH, MEM_ULTRALOW = 0, 3


def _pairs(W, workload, n, first, **kw):
    p = W.generate(workload, n, first=first, **kw)
    return [(p.pattern(i), p.text(i)) for i in range(n)]


def _batch(W, cfg, pairs):
    seqs, po, pl, to, tl = helpers.pack([a for a, _ in pairs], [b for _, b in pairs])
    al = W.Aligner(cfg)
    rc, scores, status, ops, ops_len, ops_off = al.align_batch(seqs, po, pl, to, tl)
    al.close()
    assert rc == 0
    if ops is None:  # score-only
        return [(int(status[i]), int(scores[i]), "") for i in range(len(pairs))]
    return [(int(status[i]), int(scores[i]),
             ops[ops_off[i]:ops_off[i] + ops_len[i]].tobytes().decode()) for i in range(len(pairs))]


def test_server_alone_vs_mix_and_batch_parity(gpu_available, wfa, oracle_mod):
    W, O = wfa, oracle_mod
    cfg = W.Config()
    probe = _pairs(W, 4, 24, first=500)
    others = _pairs(W, 1, 400, first=9000)
    # back-trace budget 64 KiB: the larger probes exceed it and are re-run in BiWFA mode
    srv = W.Server(cfg, backtrace_budget_bytes=64 << 10, lanes=2, batch_window_us=100,
                   biwfa_min_length=12000)

    alone = {}
    for i, (a, b) in enumerate(probe):
        rid = srv.submit(a, b)
        r = srv.wait_all([rid])[rid]
        alone[i] = r[1:5]

    # mix: probes interleaved with other requests submitted from two threads
    ids = {}
    lock = threading.Lock()

    def feed(items):
        for tag, (a, b) in items:
            rid = srv.submit(a, b)
            with lock:
                ids[tag] = rid
    mixed = [(("o", j), others[j]) for j in range(len(others))]
    for i in range(len(probe)):
        mixed.insert(i * 17, (("p", i), probe[i]))
    t1 = threading.Thread(target=feed, args=(mixed[0::2],))
    t2 = threading.Thread(target=feed, args=(mixed[1::2],))
    t1.start(); t2.start(); t1.join(); t2.join()
    got = srv.wait_all(list(ids.values()))
    assert srv.launches > 0
    srv.close()

    in_mix = {i: got[ids[("p", i)]][1:5] for i in range(len(probe))}
    assert in_mix == alone

    modes = [alone[i][2] for i in range(len(probe))]
    assert MEM_HIGH in modes and MEM_ULTRALOW in modes, modes
    hi = _batch(W, cfg, probe)
    ul = _batch(W, W.Config(memory_mode=MEM_ULTRALOW), probe)
    for i in range(len(probe)):
        st, sc, mode, ops = alone[i]
        ref = hi[i] if mode == MEM_HIGH else ul[i]
        assert (st, sc, ops) == ref, (i, mode)
    # the other requests equal the batch path as well
    ob = _batch(W, cfg, others)
    ou = None
    for j in range(len(others)):
        st, sc, mode, ops = got[ids[("o", j)]][1:5]
        if mode == MEM_HIGH:
            assert (st, sc, ops) == ob[j], j
        else:
            ou = ou or _batch(W, W.Config(memory_mode=MEM_ULTRALOW), others)
            assert (st, sc, ops) == ou[j], j

    # and the CPU checker agrees with the served results, in their modes
    pats = [a for a, _ in probe]
    txts = [b for _, b in probe]
    b = O.PairBatch.from_lists(pats, txts)
    r_hi = O.align(b, O.Penalties())
    r_ul = O.align(b, O.Penalties(), memory_mode=MEM_ULTRALOW)
    for i in range(len(probe)):
        st, sc, mode, ops = alone[i]
        r = r_hi if mode == MEM_HIGH else r_ul
        assert (st, sc, ops) == (int(r.status[i]), int(r.score[i]), r.cigar(i)), i


def test_server_score_only(gpu_available, wfa):
    W = wfa
    cfg = W.Config(score_only=True)
    pairs = _pairs(W, 1, 300, first=4)
    srv = W.Server(cfg)
    rids = [srv.submit(a, b) for a, b in pairs]
    got = srv.wait_all(rids)
    srv.close()
    ref = _batch(W, cfg, pairs)
    for i, rid in enumerate(rids):
        assert got[rid][1:3] == ref[i][:2], i


def test_server_rejects_unserved_configuration(gpu_available, wfa):
    W = wfa
    with pytest.raises(RuntimeError):
        W.Server(W.Config(memory_mode=MEM_ULTRALOW))

"""The checker against the reference library on seeded random configurations.

Each configuration draws a metric and penalties, a memory mode (high or
ultralow), a scope, an alignment form (end-to-end, ends-free lengths,
extension), a heuristic strategy set with its parameters, a step limit and a
pair workload.  The checker (oracle/) and the unmodified reference library,
compiled from its sources into oracle/_ref/, align the same pairs; scores,
statuses, CIGARs and end positions must be equal on every pair the checker
does not flag (a back-trace through a wavefront a cut emptied, or a score past
the reference's wavefront table, where it exits).  Configurations the checker
refuses are skipped.  Runs only where the reference library was built."""
import os
import random

import pytest

import helpers  # noqa: F401  (puts the repository on sys.path)


def _config(rng):
    m = rng.choice([0, 1, 2, 3, 3, 4])
    if m <= 1:
        pen = {}
    elif m == 2:
        pen = dict(match=rng.choice([0, 0, -1]), mismatch=rng.randint(2, 6),
                   gap_opening1=rng.randint(1, 4))
    elif m == 3:
        pen = dict(match=rng.choice([0, 0, -1, -2]), mismatch=rng.randint(2, 6),
                   gap_opening1=rng.randint(0, 8), gap_extension1=rng.randint(1, 3))
    else:
        pen = dict(match=rng.choice([0, 0, -1]), mismatch=rng.randint(2, 6),
                   gap_opening1=rng.randint(0, 8), gap_extension1=rng.randint(2, 4),
                   gap_opening2=rng.randint(10, 30), gap_extension2=1)
    mm = rng.choice([0, 0, 0, 3])
    so = rng.random() < 0.4
    form = None
    if mm == 0 and rng.random() < 0.4:
        form = ("extension" if rng.random() < 0.3
                else tuple(rng.choice([0, 0, 5, 20, 60]) for _ in range(4)))
    hs = None
    if rng.random() < 0.55:
        st = 0
        if rng.random() < 0.5:
            st |= rng.choice([0x04, 0x40])
        if rng.random() < 0.4 and m >= 2:
            st |= rng.choice([0x10, 0x20] if mm == 0 else [0x10])
        if rng.random() < 0.4:
            st |= rng.choice([0x01, 0x02])
        if st:
            hs = dict(strategy=st, min_wavefront_length=rng.choice([1, 10, 20]),
                      max_distance_threshold=rng.choice([0, 10, 50]),
                      steps_between_cutoffs=rng.choice([1, 2, 3]),
                      xdrop=rng.choice([20, 50, 100]), zdrop=rng.choice([20, 50, 100]),
                      min_k=-rng.choice([5, 20, 40]), max_k=rng.choice([5, 20, 40]))
    ms = rng.choice([0, 0, 200, 1000, 3000])
    if m <= 1 and hs and ms == 0:
        ms = 3000  # edit/indel runs on past null wavefronts: the reference needs a limit
    wl = rng.choice([0, 1, 1, 5, 6])
    n = {0: 40, 1: 16, 5: 10, 6: 16}[wl]
    pa, pb = ((rng.choice([300, 800, 2000]), rng.choice([50, 150, 300])) if wl == 5 else (0, 0))
    return m, pen, form, hs, mm, so, ms, wl, n, rng.randint(0, 10 ** 6), pa, pb


_RNG = random.Random(3)
CONFIGS = [_config(_RNG) for _ in range(60)]


@pytest.mark.parametrize("idx", range(len(CONFIGS)))
def test_checker_matches_reference_on_random_configuration(oracle_mod, wfa, idx):
    O, W = oracle_mod, wfa
    if not os.path.exists(O.REF_SCALAR_LIB):
        pytest.skip("the reference library is not built here")
    m, pen, form, hs, mm, so, ms, wl, n, first, pa, pb = CONFIGS[idx]
    p = W.generate(wl, n, first=first, param=pa, param2=pb)
    b = O.PairBatch(p.seqs, p.p_off, p.p_len, p.t_off, p.t_len)
    penalties = O.Penalties(metric=m, **pen)
    h = O.Heuristic(**hs) if hs else None
    try:
        a = O.align(b, penalties, memory_mode=mm, score_only=so, form=form, heuristic=h,
                    max_steps=ms)
    except ValueError:
        pytest.skip("a configuration the checker refuses")
    keep = [i for i in range(b.n)
            if not (a.flags[i] & (O.FLAG_STALE_SOURCE | O.FLAG_OVER_BOUND))]
    if not keep:
        return
    sub = O.PairBatch.from_lists([b.pattern(i) for i in keep], [b.text(i) for i in keep])
    r = O.align(sub, penalties, memory_mode=mm, score_only=so, form=form, heuristic=h,
                max_steps=ms, kind="reference_scalar")
    for j, i in enumerate(keep):
        got = (int(a.score[i]), int(a.status[i]), a.cigar(i), int(a.end[i][0]),
               int(a.end[i][1]))
        want = (int(r.score[j]), int(r.status[j]), r.cigar(j), int(r.end[j][0]),
                int(r.end[j][1]))
        assert got == want, (CONFIGS[idx], i)

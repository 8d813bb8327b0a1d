"""Match starts found on the device against the oracle's first_match.

For every hit the CPU matcher reports MatchResult(start, target_end + 1); the
start comes from a reverse pass (semi_global_aln_start_end / ssw_align).  The
device runs that pass for all hits at once (ish_gpu_match_starts); starts must
be identical, record by record, for every end-freeness configuration.
"""
import os

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.matcher import StripedLocalMatcher, StripedSemiGlobalMatcher
from ish_gb300.scoring import ScoringMatrix

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.close()


def planted(rng, alphabet, q, n, lmin, lmax, frac=0.4, sub=0.15, indel=0.03):
    recs = []
    for _ in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        r = list(rng.integers(0, alphabet, L, dtype=np.uint8))
        if len(q) and rng.random() < frac:
            cp = []
            for c in q:
                x = rng.random()
                if x < indel / 2:
                    continue
                cp.append(int(rng.integers(0, alphabet)) if x < indel / 2 + sub else int(c))
                if rng.random() < indel / 2:
                    cp.append(int(rng.integers(0, alphabet)))
            pos = int(rng.integers(0, L + 1))
            r[pos:pos] = cp
        recs.append(np.array(r, np.uint8))
    return recs


def check(ctx, algo, kind, q, recs, gap_open, gap_ext, ends, thr):
    m = ScoringMatrix(kind)
    mx = int(m.values[q, q].astype(np.int64).sum()) if len(q) else 0
    buf, off = native.pack_records(recs)
    qid = ctx.set_query(q, kind, m.values, algo, gap_open, gap_ext, ends, mx, thr)
    sid = ctx.records_load(buf, off)
    try:
        g = ctx.score_set(qid, sid)
        starts = ctx.match_starts(qid, sid, g["hit_idx"], g["tend"][g["hit_idx"]])
    finally:
        ctx.records_free(sid)
        ctx.free_query(qid)
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, kind, q, mx, thr,
                   gap_open=gap_open, gap_extend=gap_ext, ends=ends)
    o = om.batch(buf, off, threads=THREADS)
    hits = np.nonzero(o["hit"])[0]
    assert np.array_equal(g["hit_idx"], hits), "hit sets differ"
    bad = np.nonzero(starts != o["start"][hits])[0]
    assert len(bad) == 0, (f"{len(bad)}/{len(hits)} starts differ; first record {hits[bad[0]]}: gpu {starts[bad[0]]} "
                           f"oracle {o['start'][hits[bad[0]]]}")
    assert np.array_equal(g["tend"][hits] + 1, o["end"][hits])
    return len(hits)


@pytest.mark.parametrize("ends", list(range(16)))
def test_semi_global_starts_all_ends(ctx, ends):
    rng = np.random.default_rng(700 + ends)
    q = rng.integers(0, 5, 60, dtype=np.uint8)
    recs = planted(rng, 5, q, 300, 0, 250)
    n = check(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, q, recs, 3, 1, ends, 0.3)
    assert n > 0


@pytest.mark.parametrize("qlen", [1, 9, 40, 150, 333])
@pytest.mark.parametrize("kind", [O.ACTGN0, O.BLOSUM62])
def test_local_starts(ctx, qlen, kind):
    rng = np.random.default_rng(800 + qlen + kind)
    alpha = 5 if kind == O.ACTGN0 else 20
    q = rng.integers(0, alpha, qlen, dtype=np.uint8)
    recs = planted(rng, alpha, q, 250, 0, 2 * qlen + 80)
    check(ctx, native.ALGO_LOCAL, kind, q, recs, 10 if kind == O.BLOSUM62 else 3, 1, 0, 0.3)


@pytest.mark.parametrize("qlen", [24, 300, 700])
def test_protein_semi_global_starts(ctx, qlen):
    rng = np.random.default_rng(900 + qlen)
    q = rng.integers(0, 20, qlen, dtype=np.uint8)
    recs = planted(rng, 20, q, 200, 10, 3 * qlen)
    for ends in (12, 15, 3, 0):
        check(ctx, native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, recs, 10, 1, ends, 0.4)


def test_starts_with_empty_records_and_zero_threshold(ctx):
    # threshold 0: empty records are semi-global hits too; their prefix is
    # empty and the start is -1, as the CPU matcher reports
    rng = np.random.default_rng(901)
    q = rng.integers(65, 69, 12, dtype=np.uint8)
    recs = [rng.integers(65, 69, int(rng.integers(0, 40)), dtype=np.uint8) for _ in range(150)]
    recs += [np.zeros(0, np.uint8)] * 3
    for ends in (12, 15, 0, 4, 8):
        check(ctx, native.ALGO_SEMI_GLOBAL, O.ASCII, q, recs, 3, 1, ends, 0.0)


def test_matchers_report_match_results(ctx):
    rng = np.random.default_rng(902)
    pat = b"GATTACAGATTACACCGT"
    lines = [bytes(rng.choice(list(b"ACGT"), int(rng.integers(5, 80)))) for _ in range(200)]
    lines = [l[:10] + pat + l[10:] if i % 5 == 0 else l for i, l in enumerate(lines)]
    for mt, om in ((StripedSemiGlobalMatcher(pat, 0.8, "FFTT", "actgn", context=ctx),
                    O.Matcher.from_ascii(O.SEMI_GLOBAL, O.ACTGN, pat, 0.8, ends=O.TS | O.TE)),
                   (StripedLocalMatcher(pat, 0.8, "actgn", context=ctx),
                    O.Matcher.from_ascii(O.LOCAL, O.ACTGN, pat, 0.8))):
        enc = [mt.convert_ascii_to_encoding(l) for l in lines]
        res = mt.batch_match(enc)
        want = []
        for i, e in enumerate(enc):
            m = om.first_match(e)
            if m is not None:
                want.append((i, m[0], m[1]))
        assert res.matches() == want
        assert len(want) >= 30


@pytest.mark.parametrize("ends", [12, 13])
def test_starts_in_long_records(ctx, ends):
    # hits deep inside long records: the reverse pass over their prefixes is
    # windowed like a forward pass, starts must still be the CPU matcher's
    rng = np.random.default_rng(950 + ends)
    q = rng.integers(0, 5, 80, dtype=np.uint8)
    recs = planted(rng, 5, q, 60, 50, 400, frac=0.3)
    for L in (150_000, 90_000, 40_000):
        r = rng.integers(0, 5, L, dtype=np.uint8)
        for pos in (int(L * 0.9), int(L * 0.4)):
            cp = q.copy()
            mut = rng.random(len(cp)) < 0.05
            cp[mut] = rng.integers(0, 5, int(mut.sum()), dtype=np.uint8)
            r[pos:pos + len(cp)] = cp
        recs.append(r)
    n = check(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, q, recs, 3, 1, ends, 0.5)
    assert n >= 3

"""Long records scored as overlapping windows.

When a set's longest records would bound the pass, the engine cuts them into
windows that overlap by more than any best alignment can span and folds the
window results per record.  The results must be bit-identical to the oracle
and to whole-record scoring (ISH_OPT_WINDOWS = 0), including the first-row /
smallest-column tie rules when the maximum occurs in several windows.
"""
import os

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import ScoringMatrix

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.set_option(native.OPT_WINDOWS, 1)
    c.close()


def long_records(rng, alphabet, q, n_short, long_lens, every, sub=0.0):
    """Short random records plus a few long ones carrying a copy of the query
    every `every` rows (exact copies when sub == 0: the maximum ties)."""
    recs = [rng.integers(0, alphabet, int(rng.integers(1, 400)), dtype=np.uint8) for _ in range(n_short)]
    for L in long_lens:
        r = rng.integers(0, alphabet, L, dtype=np.uint8)
        pos = int(rng.integers(0, every))
        while pos + len(q) <= L:
            cp = q.copy()
            if sub:
                mut = rng.random(len(cp)) < sub
                cp[mut] = rng.integers(0, alphabet, int(mut.sum()), dtype=np.uint8)
            r[pos:pos + len(cp)] = cp
            pos += every + int(rng.integers(0, every // 3 + 1))
        recs.append(r)
    order = rng.permutation(len(recs))
    return [recs[i] for i in order]


def score(ctx, algo, kind, q, buf, off, gap_open, gap_ext, ends, windows):
    m = ScoringMatrix(kind)
    mx = int(m.values[q, q].astype(np.int64).sum())
    ctx.set_option(native.OPT_WINDOWS, windows)
    qid = ctx.set_query(q, kind, m.values, algo, gap_open, gap_ext, ends, mx, 0.5)
    try:
        sid = ctx.records_load(buf, off)
        try:
            r = ctx.score_set(qid, sid)
            nwin = ctx.last_windows()
        finally:
            ctx.records_free(sid)
    finally:
        ctx.free_query(qid)
        ctx.set_option(native.OPT_WINDOWS, 1)
    return r, nwin


def oracle(algo, kind, q, buf, off, gap_open, gap_ext, ends):
    m = ScoringMatrix(kind)
    mx = int(m.values[q, q].astype(np.int64).sum())
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, kind, q, mx, 0.5,
                   gap_open=gap_open, gap_extend=gap_ext, ends=ends)
    return om.batch(buf, off, threads=THREADS)


def same(a, b, label):
    for k in ("score", "qend", "tend", "hit"):
        bad = np.nonzero(np.asarray(a[k]) != np.asarray(b[k]))[0]
        assert len(bad) == 0, f"{label}: {k} differs on {len(bad)} records, first #{bad[0]}: {a[k][bad[0]]} vs {b[k][bad[0]]}"


CASES = [
    # (algo, ends)
    (native.ALGO_SEMI_GLOBAL, 12),  # free target start and end
    (native.ALGO_SEMI_GLOBAL, 13),  # ... and free query start
    (native.ALGO_LOCAL, 0),
]


@pytest.mark.parametrize("algo,ends", CASES)
@pytest.mark.parametrize("sub", [0.0, 0.12])
def test_windows_equal_oracle_and_whole_records(ctx, algo, ends, sub):
    rng = np.random.default_rng(61 + ends + int(sub * 100))
    q = rng.integers(0, 20, 100, dtype=np.uint8)
    recs = long_records(rng, 20, q, 300, [230_000, 180_017, 96_000, 41_003], every=2500, sub=sub)
    buf, off = native.pack_records(recs)
    g, nwin = score(ctx, algo, O.BLOSUM62, q, buf, off, 10, 1, ends, 1)
    assert nwin > len(recs), "the long records were not windowed"
    whole, n0 = score(ctx, algo, O.BLOSUM62, q, buf, off, 10, 1, ends, 0)
    assert n0 == 0
    same(g, whole, f"windows vs whole records algo={algo} ends={ends}")
    same(g, oracle(algo, O.BLOSUM62, q, buf, off, 10, 1, ends), f"windows vs oracle algo={algo} ends={ends}")


@pytest.mark.parametrize("algo", [native.ALGO_SEMI_GLOBAL, native.ALGO_LOCAL])
def test_windows_ties_small_alphabet(ctx, algo):
    # four letters, many equal scores across windows
    rng = np.random.default_rng(67)
    q = rng.integers(65, 69, 30, dtype=np.uint8)
    recs = [rng.integers(65, 69, int(rng.integers(0, 200)), dtype=np.uint8) for _ in range(200)]
    recs += [rng.integers(65, 69, L, dtype=np.uint8) for L in (120_000, 77_777)]
    buf, off = native.pack_records(recs)
    ends = 12 if algo == native.ALGO_SEMI_GLOBAL else 0
    g, nwin = score(ctx, algo, O.ASCII, q, buf, off, 3, 1, ends, 1)
    assert nwin > len(recs)
    same(g, oracle(algo, O.ASCII, q, buf, off, 3, 1, ends), f"ascii ties algo={algo}")


@pytest.mark.parametrize("ends", [15, 0, 8])
def test_no_windows_when_the_span_is_unbounded(ctx, ends):
    # a fixed target start, or a free query end, gives no span bound: the
    # long records are scored whole
    rng = np.random.default_rng(71 + ends)
    q = rng.integers(0, 20, 60, dtype=np.uint8)
    recs = long_records(rng, 20, q, 100, [150_000], every=4000, sub=0.1)
    buf, off = native.pack_records(recs)
    g, nwin = score(ctx, native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, buf, off, 10, 1, ends, 1)
    assert nwin == 0
    same(g, oracle(native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, buf, off, 10, 1, ends), f"ends={ends}")


@pytest.mark.parametrize("algo,ends", CASES)
@pytest.mark.parametrize("gaps", [(10, 1), (207, 200)])
def test_windows_invent_no_alignment(ctx, algo, ends, gaps):
    # random records with no copy of the query: the best score of a record is
    # small, so a window that let an alignment begin where the whole record
    # does not (a free query start past row 0) would show up as a larger
    # score at a later row
    rng = np.random.default_rng(73 + ends + gaps[1])
    q = rng.integers(0, 20, 30, dtype=np.uint8)
    recs = [rng.integers(0, 20, int(rng.integers(1, 300)), dtype=np.uint8) for _ in range(150)]
    recs += [rng.integers(0, 20, L, dtype=np.uint8) for L in (60_000, 31_111, 9_000)]
    buf, off = native.pack_records(recs)
    g, nwin = score(ctx, algo, O.BLOSUM62, q, buf, off, gaps[0], gaps[1], ends, 1)
    assert nwin > len(recs)
    same(g, oracle(algo, O.BLOSUM62, q, buf, off, gaps[0], gaps[1], ends), f"algo={algo} ends={ends} gaps={gaps}")

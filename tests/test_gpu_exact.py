"""The exact kernels: the reference's striped passes emulated lane by lane.

Outside the regime where the wavefront kernels are exact -- gap_open <=
gap_extend, int16 boundary rows that wrap, queries longer than the wavefront
shapes, or on request (ISH_KERNEL_EXACT) -- the engine runs these; results
must equal the oracle (the reference's algorithm restated on the CPU) for the
same lane counts, bit for bit.
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
    c.close()


def recs_with_copies(rng, alpha, q, n, lmin, lmax, frac=0.3, sub=0.1):
    out = []
    for _ in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        r = rng.integers(0, alpha, L, dtype=np.uint8)
        if len(q) and L >= len(q) and rng.random() < frac:
            pos = int(rng.integers(0, L - len(q) + 1))
            cp = q.copy()
            m = rng.random(len(cp)) < sub
            cp[m] = rng.integers(0, alpha, int(m.sum()), dtype=np.uint8)
            r[pos:pos + len(cp)] = cp
        out.append(r)
    return out


def both(ctx, algo, kind, q, recs, gap_open, gap_ext, ends, thr=0.4, lanes=(8, 16, 8), kernel=native.KERNEL_AUTO):
    m = ScoringMatrix(kind)
    mx = int(m.values[q, q].astype(np.int64).sum()) if len(q) else 0
    buf, off = native.pack_records(recs)
    ctx.set_option(native.OPT_KERNEL, kernel)
    ctx.set_option(native.OPT_SG_LANES, lanes[0])
    ctx.set_option(native.OPT_SW_U8_LANES, lanes[1])
    ctx.set_option(native.OPT_SW_U16_LANES, lanes[2])
    qid = ctx.set_query(q, kind, m.values, algo, gap_open, gap_ext, ends, mx, thr)
    try:
        g = ctx.score(qid, buf, off)
    finally:
        ctx.free_query(qid)
        ctx.set_option(native.OPT_KERNEL, native.KERNEL_AUTO)
        ctx.set_option(native.OPT_SG_LANES, 8)
        ctx.set_option(native.OPT_SW_U8_LANES, 16)
        ctx.set_option(native.OPT_SW_U16_LANES, 8)
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, kind, q, mx, thr,
                   gap_open=gap_open, gap_extend=gap_ext, ends=ends, w_sg=lanes[0], w_u8=lanes[1], w_u16=lanes[2])
    o = om.batch(buf, off, threads=THREADS)
    for k in ("score", "qend", "tend", "hit"):
        bad = np.nonzero(g[k] != o[k])[0]
        assert len(bad) == 0, (f"{k} differs on {len(bad)}/{len(recs)}; first #{bad[0]}: gpu "
                               f"({g['score'][bad[0]]},{g['qend'][bad[0]]},{g['tend'][bad[0]]},{g['hit'][bad[0]]}) "
                               f"oracle ({o['score'][bad[0]]},{o['qend'][bad[0]]},{o['tend'][bad[0]]},{o['hit'][bad[0]]})")
    return g


@pytest.mark.parametrize("gaps", [(1, 1), (2, 2), (1, 2), (0, 1)])
@pytest.mark.parametrize("kind", [O.ACTGN, O.BLOSUM62])
def test_open_not_above_extend(ctx, gaps, kind):
    rng = np.random.default_rng(5000 + 10 * gaps[0] + gaps[1] + kind)
    alpha = 5 if kind == O.ACTGN else 20
    for qlen in (7, 40, 130):
        q = rng.integers(0, alpha, qlen, dtype=np.uint8)
        recs = recs_with_copies(rng, alpha, q, 80, 0, 2 * qlen + 30)
        for ends in (0, 3, 5, 10, 12, 15):
            both(ctx, native.ALGO_SEMI_GLOBAL, kind, q, recs, gaps[0], gaps[1], ends)
        both(ctx, native.ALGO_LOCAL, kind, q, recs, gaps[0], gaps[1], 0)


@pytest.mark.parametrize("lanes", [(8, 16, 8), (16, 32, 16), (32, 8, 32)])
def test_lane_counts_of_other_hosts(ctx, lanes):
    # an AVX2 host runs 16 int16 / 32 uint8 lanes; results outside the exact
    # regime follow the lane count
    rng = np.random.default_rng(5100 + lanes[0])
    q = rng.integers(0, 20, 90, dtype=np.uint8)
    recs = recs_with_copies(rng, 20, q, 80, 10, 300)
    for ends in (12, 15):
        both(ctx, native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, recs, 1, 1, ends, lanes=lanes)
    both(ctx, native.ALGO_LOCAL, O.BLOSUM62, q, recs, 1, 1, 0, lanes=lanes)


@pytest.mark.parametrize("algo", [native.ALGO_SEMI_GLOBAL, native.ALGO_LOCAL])
def test_forced_exact_kernel_in_the_fast_regime(ctx, algo):
    rng = np.random.default_rng(5200 + algo)
    q = rng.integers(0, 20, 150, dtype=np.uint8)
    recs = recs_with_copies(rng, 20, q, 150, 0, 400)
    for ends in ((12, 15, 0) if algo == native.ALGO_SEMI_GLOBAL else (0,)):
        fast = both(ctx, algo, O.BLOSUM62, q, recs, 10, 1, ends)
        ex = both(ctx, algo, O.BLOSUM62, q, recs, 10, 1, ends, kernel=native.KERNEL_EXACT)
        for k in ("score", "qend", "tend", "hit"):
            assert np.array_equal(fast[k], ex[k])


def test_local_uint8_saturation_reruns_with_uint16(ctx):
    # high-identity copies of a long query: scores beyond 255 - bias send the
    # uint8 pass into saturation and the record is rerun with uint16 lanes
    rng = np.random.default_rng(5300)
    q = rng.integers(0, 20, 200, dtype=np.uint8)
    recs = recs_with_copies(rng, 20, q, 60, 150, 600, frac=0.6, sub=0.02)
    g = both(ctx, native.ALGO_LOCAL, O.BLOSUM62, q, recs, 1, 1, 0)
    assert (g["score"] > 255).sum() > 5


def test_wrapped_boundary_rows(ctx):
    # non-free target start with records long enough that the int16 boundary
    # row -open - ext * (i - 1) wraps: the reference's lanes see wrapped values
    rng = np.random.default_rng(5400)
    q = rng.integers(0, 5, 30, dtype=np.uint8)
    recs = [rng.integers(0, 5, L, dtype=np.uint8) for L in (40000, 33000, 70000, 120, 5)]
    for ends in (0, 3, 8, 11):
        both(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, q, recs, 3, 1, ends)


def test_query_longer_than_wavefront_shapes(ctx):
    rng = np.random.default_rng(5500)
    q = rng.integers(0, 5, 2300, dtype=np.uint8)
    recs = recs_with_copies(rng, 5, q, 20, 100, 3000)
    both(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, q, recs, 3, 1, 12)
    both(ctx, native.ALGO_LOCAL, O.ACTGN, q, recs, 3, 1, 0)


def test_match_starts_outside_the_fast_regime(ctx):
    # the reverse pass of start finding runs on the exact kernels too
    rng = np.random.default_rng(5600)
    m = ScoringMatrix(O.BLOSUM62)
    q = rng.integers(0, 20, 60, dtype=np.uint8)
    recs = recs_with_copies(rng, 20, q, 150, 0, 300, frac=0.5)
    buf, off = native.pack_records(recs)
    mx = int(m.values[q, q].sum())
    for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 15), (native.ALGO_LOCAL, 0)):
        qid = ctx.set_query(q, O.BLOSUM62, m.values, algo, 2, 2, ends, mx, 0.3)
        sid = ctx.records_load(buf, off)
        try:
            g = ctx.score_set(qid, sid)
            st = ctx.match_starts(qid, sid, g["hit_idx"], g["tend"][g["hit_idx"]])
        finally:
            ctx.records_free(sid)
            ctx.free_query(qid)
        om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, O.BLOSUM62, q, mx, 0.3,
                       gap_open=2, gap_extend=2, ends=ends)
        o = om.batch(buf, off, threads=THREADS)
        hits = np.nonzero(o["hit"])[0]
        assert np.array_equal(g["hit_idx"], hits) and len(hits) > 10
        assert np.array_equal(st, o["start"][hits])

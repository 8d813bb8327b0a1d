"""Batched multi-query launches (ish_gpu_score_multi) and the autotuner.

Every query of a batched launch must give exactly what the single-query path
gives for it (ish_gpu_score_set) and what the oracle gives: the same integer
scores, end coordinates, hit flags and hit lists.  The launch is a CUDA graph
replayed on later calls, so repeated calls must agree too.
"""
import ctypes as C
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


def records(rng, alphabet, n, lmin, lmax, plants=(), plant_frac=0.05):
    out = []
    for _ in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        r = rng.integers(0, alphabet, L, dtype=np.uint8)
        if plants and rng.random() < plant_frac:
            q = plants[int(rng.integers(0, len(plants)))]
            if 0 < len(q) <= L:
                pos = int(rng.integers(0, L - len(q) + 1))
                cp = q.copy()
                mut = rng.random(len(cp)) < 0.1
                cp[mut] = rng.integers(0, alphabet, int(mut.sum()), dtype=np.uint8)
                r[pos:pos + len(cp)] = cp
        out.append(r)
    return out


def make_queries(ctx, kind, specs, rng, alphabet, gap_open, gap_ext, thr=0.5):
    m = ScoringMatrix(kind)
    qs, ids = [], []
    for qlen, algo, ends in specs:
        q = rng.integers(0, alphabet, qlen, dtype=np.uint8)
        mx = int(m.values[q, q].astype(np.int64).sum()) if qlen else 0
        ids.append(ctx.set_query(q, kind, m.values, algo, gap_open, gap_ext, ends, mx, thr))
        qs.append((q, algo, ends, mx))
    return qs, ids


def check_against_single(ctx, ids, sid, res):
    for i, qid in enumerate(ids):
        one = ctx.score_set(qid, sid)
        for k in ("score", "qend", "tend", "hit"):
            bad = np.nonzero(res[k][i] != one[k])[0]
            assert len(bad) == 0, f"query #{i}: {k} differs from score_set on {len(bad)} records (first {bad[:3]})"
        assert np.array_equal(res["hit_idx"][i], one["hit_idx"]), f"query #{i}: hit list differs"


def check_against_oracle(kind, qs, buf, off, res, gap_open, gap_ext, thr=0.5):
    for i, (q, algo, ends, mx) in enumerate(qs):
        om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, kind, q, mx, thr,
                       gap_open=gap_open, gap_extend=gap_ext, ends=ends)
        o = om.batch(buf, off, threads=THREADS)
        for k in ("score", "qend", "tend", "hit"):
            bad = np.nonzero(res[k][i] != o[k])[0]
            assert len(bad) == 0, (f"query #{i} (Q={len(q)}, algo={algo}, ends={ends}): {k} differs from the "
                                   f"oracle on {len(bad)} records (first {bad[:3]})")
        assert np.array_equal(res["hit_idx"][i], np.nonzero(o["hit"])[0])


def test_multi_nucleotide_mixed_lengths_and_algorithms(ctx):
    rng = np.random.default_rng(31)
    specs = [(1, native.ALGO_SEMI_GLOBAL, 12), (7, native.ALGO_LOCAL, 0), (30, native.ALGO_SEMI_GLOBAL, 15),
             (50, native.ALGO_SEMI_GLOBAL, 12), (120, native.ALGO_LOCAL, 0), (260, native.ALGO_SEMI_GLOBAL, 0),
             (333, native.ALGO_SEMI_GLOBAL, 5), (500, native.ALGO_SEMI_GLOBAL, 12), (800, native.ALGO_LOCAL, 0),
             (1000, native.ALGO_SEMI_GLOBAL, 12)]
    qs, ids = make_queries(ctx, O.ACTGN, specs, rng, 5, 3, 1)
    recs = records(rng, 5, 1500, 0, 400, plants=[q for q, *_ in qs])
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        res = ctx.score_multi(ids, sid)
        check_against_oracle(O.ACTGN, qs, buf, off, res, 3, 1)
        check_against_single(ctx, ids, sid, res)
        again = ctx.score_multi(ids, sid)  # graph replay
        for k in ("score", "qend", "tend", "hit"):
            assert np.array_equal(again[k], res[k])
        assert sum(len(h) for h in res["hit_idx"]) > 0
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_multi_protein_duplicates_and_empty_query(ctx):
    rng = np.random.default_rng(32)
    specs = [(300, native.ALGO_SEMI_GLOBAL, 12), (300, native.ALGO_LOCAL, 0), (0, native.ALGO_SEMI_GLOBAL, 12),
             (90, native.ALGO_LOCAL, 0), (700, native.ALGO_SEMI_GLOBAL, 10)]
    qs, ids = make_queries(ctx, O.BLOSUM62, specs, rng, 20, 10, 1)
    recs = records(rng, 20, 800, 0, 900, plants=[q for q, *_ in qs if len(q)])
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        order = [ids[0], ids[1], ids[0], ids[2], ids[3], ids[4], ids[1]]
        res = ctx.score_multi(order, sid)
        check_against_single(ctx, order, sid, res)
        sel = [0, 1, 2, 3, 4]
        check_against_oracle(O.BLOSUM62, [qs[i] for i in sel], buf, off,
                             {k: (v[[0, 1, 3, 4, 5]] if k != "hit_idx" else [v[j] for j in (0, 1, 3, 4, 5)])
                              for k, v in res.items()}, 10, 1)
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_multi_large_set(ctx):
    # enough records that every block works on several queries
    rng = np.random.default_rng(33)
    specs = [(60, native.ALGO_SEMI_GLOBAL, 12), (61, native.ALGO_SEMI_GLOBAL, 12), (150, native.ALGO_LOCAL, 0),
             (400, native.ALGO_SEMI_GLOBAL, 12)]
    qs, ids = make_queries(ctx, O.ACTGN, specs, rng, 5, 3, 1)
    n = 120_000
    lens = rng.integers(100, 301, n)
    flat = rng.integers(0, 5, int(lens.sum()), dtype=np.uint8)
    off = np.zeros(n + 1, np.uint64)
    off[1:] = np.cumsum(lens)
    sid = ctx.records_load(flat, off)
    try:
        res = ctx.score_multi(ids, sid, want=("score", "qend", "tend", "hit", "hit_idx"))
        check_against_single(ctx, ids, sid, res)
        sub = np.arange(0, n, 97)
        sb, so = native.pack_records([flat[int(off[i]):int(off[i + 1])] for i in sub])
        check_against_oracle(O.ACTGN, qs, sb, so, {k: (v[:, sub] if k != "hit_idx" else None)
                                                   for k, v in res.items() if k != "hit_idx"} |
                             {"hit_idx": [np.nonzero(res["hit"][i, sub])[0] for i in range(len(ids))]}, 3, 1)
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_multi_hits_overflow_and_invalidation(ctx):
    rng = np.random.default_rng(34)
    qs, ids = make_queries(ctx, O.ACTGN, [(20, native.ALGO_SEMI_GLOBAL, 15), (25, native.ALGO_LOCAL, 0)], rng, 5,
                           3, 1, thr=0.0)
    recs = records(rng, 5, 300, 30, 60)
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    L = native.load()
    try:
        q = np.array(ids, np.int32)
        idx = np.zeros(4, np.uint32)
        offs = np.zeros(3, np.uint64)
        rc = L.ish_gpu_score_multi(ctx._h, q.ctypes.data_as(C.POINTER(C.c_int32)), 2, sid, None, None, None, None,
                                   idx.ctypes.data_as(C.POINTER(C.c_uint32)), 4,
                                   offs.ctypes.data_as(C.POINTER(C.c_uint64)))
        assert rc == native.EOVERFLOW
        full = ctx.score_multi(ids, sid)
        assert offs[2] == sum(len(h) for h in full["hit_idx"]) > 4
        assert offs[1] == len(full["hit_idx"][0])
        # freeing a query drops the cached launch; the survivors still run
        ctx.free_query(ids[1])
        only = ctx.score_multi(ids[:1], sid)
        assert np.array_equal(only["score"][0], full["score"][0])
        with pytest.raises(native.IshGpuError):
            ctx.score_multi(ids, sid)
    finally:
        ctx.records_free(sid)
        ctx.free_query(ids[0])
    with pytest.raises(native.IshGpuError):
        ctx.score_multi(ids[:1], sid)


def test_autotune_changes_shapes_not_results(ctx):
    rng = np.random.default_rng(35)
    specs = [(40, native.ALGO_SEMI_GLOBAL, 12), (300, native.ALGO_LOCAL, 0), (640, native.ALGO_SEMI_GLOBAL, 12)]
    qs, ids = make_queries(ctx, O.BLOSUM62, specs, rng, 20, 10, 1)
    recs = records(rng, 20, 4000, 50, 500, plants=[q for q, *_ in qs])
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        before = ctx.score_multi(ids, sid)
        g, k = ctx.autotune(sid, ids)
        for (q, *_), gg, kk in zip(qs, g, k):
            assert gg in (1, 2, 4, 8, 16, 32) and gg * kk >= len(q) + 1
        after = ctx.score_multi(ids, sid)
        for key in ("score", "qend", "tend", "hit"):
            assert np.array_equal(before[key], after[key])
        check_against_single(ctx, ids, sid, after)
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_multi_with_exact_kernel_queries(ctx):
    # queries outside the wavefront kernels' regime (gap_open <= gap_extend)
    # run on the lane-exact kernels inside the same batched launch
    rng = np.random.default_rng(36)
    m = ScoringMatrix(O.BLOSUM62)
    specs = [(80, native.ALGO_SEMI_GLOBAL, 12), (120, native.ALGO_LOCAL, 0)]
    qs, ids = make_queries(ctx, O.BLOSUM62, specs, rng, 20, 10, 1)
    qx = rng.integers(0, 20, 60, dtype=np.uint8)
    mx = int(m.values[qx, qx].sum())
    ex = [ctx.set_query(qx, O.BLOSUM62, m.values, algo, g, g, ends, mx, 0.5)
          for algo, ends, g in ((native.ALGO_SEMI_GLOBAL, 15, 1), (native.ALGO_LOCAL, 0, 2))]
    recs = records(rng, 20, 600, 0, 400, plants=[q for q, *_ in qs] + [qx])
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        order = [ids[0], ex[0], ids[1], ex[1]]
        res = ctx.score_multi(order, sid)
        check_against_single(ctx, order, sid, res)
        exq = [(qx, native.ALGO_SEMI_GLOBAL, 15, mx)]
        check_against_oracle(O.BLOSUM62, exq, buf, off, {k: (v[[1]] if k != "hit_idx" else [v[1]])
                                                           for k, v in res.items()}, 1, 1, thr=0.5)
        again = ctx.score_multi(order, sid)  # graph replay
        assert np.array_equal(again["score"], res["score"])
    finally:
        ctx.records_free(sid)
        for qid in ids + ex:
            ctx.free_query(qid)


def test_multi_windows_long_records(ctx):
    # a few 40-60 kb records among short ones: the batched launch scores the
    # long ones as overlapping windows for the queries whose fold is exact
    # (free target start, no free query start) and whole for the others; all
    # results equal the launch without windows, the single-query path and the
    # oracle, and the windowed launch runs one fold kernel per windowed query
    rng = np.random.default_rng(23)
    kind, alphabet = O.ACTGN, 5
    TS, TE, QS = native.FREE_TARGET_START, native.FREE_TARGET_END, native.FREE_QUERY_START
    specs = [(100, native.ALGO_SEMI_GLOBAL, TS | TE), (60, native.ALGO_LOCAL, 0),
             (150, native.ALGO_SEMI_GLOBAL, TS | TE | QS), (80, native.ALGO_SEMI_GLOBAL, TS | TE),
             (120, native.ALGO_LOCAL, 0)]
    qs, ids = make_queries(ctx, kind, specs, rng, alphabet, 3, 1)
    recs = records(rng, alphabet, 300, 1, 400, plants=[q for q, *_ in qs], plant_frac=0.1)
    for L in (40_000, 52_000, 60_000):
        r = rng.integers(0, alphabet, L, dtype=np.uint8)
        for q, *_ in qs:  # copies of the queries deep in the record, so hits span windows
            pos = int(rng.integers(0, L - len(q)))
            r[pos:pos + len(q)] = q
        recs.insert(int(rng.integers(0, len(recs))), r)
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        l0 = ctx.launch_count()
        res = ctx.score_multi(ids, sid)
        l1 = ctx.launch_count()
        ctx.set_option(native.OPT_WINDOWS, 0)
        whole = ctx.score_multi(ids, sid)
        l2 = ctx.launch_count()
        ctx.set_option(native.OPT_WINDOWS, 1)
        assert (l1 - l0) - (l2 - l1) == 4, ((l1 - l0), (l2 - l1))  # four windowed queries: one fold each
        for k in ("score", "qend", "tend", "hit"):
            assert np.array_equal(res[k], whole[k]), k
        for i in range(len(ids)):
            assert np.array_equal(res["hit_idx"][i], whole["hit_idx"][i])
        check_against_single(ctx, ids, sid, res)
        check_against_oracle(kind, qs, buf, off, res, 3, 1)
        # a replay of the captured plan gives the same
        again = ctx.score_multi(ids, sid)
        for k in ("score", "qend", "tend", "hit"):
            assert np.array_equal(res[k], again[k]), k
    finally:
        ctx.set_option(native.OPT_WINDOWS, 1)
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)

"""Parity on the benchmark workloads' own inputs.

Each test draws a seeded sample from one generator of ``ish_gb300.workloads``
-- the same length distributions, residue compositions, planted copies, matrix,
gap penalties and end configuration the benchmark lines are measured on -- and
requires the GPU's results to be identical to the oracle's for every record:
scores, end coordinates, hit flags and hit lists, and for the hits the match
starts of the device reverse pass (ish_gpu_match_starts).  Where the workload's
own threshold leaves no hits (the protein search: 40 %-divergent copies stay
below 0.8), the test lowers it so compaction and start finding run.

The generators are the benchmark's; only the record counts are cut so the
oracle finishes in seconds.
"""
import os

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native, workloads
from ish_gb300.scoring import ScoringMatrix

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.close()


def _max_score(kind, q):
    m = ScoringMatrix(kind)
    return int(m.values[q, q].astype(np.int64).sum())


def _oracle(wl, q, algo, ends, gap_open, gap_ext, thr):
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, wl.kind, q,
                   _max_score(wl.kind, q), thr, gap_open=gap_open, gap_extend=gap_ext, ends=ends)
    return om.batch(wl.records, wl.offsets, threads=THREADS)


def _compare(g, o, label, starts=None):
    n = len(o["score"])
    for k in ("score", "qend", "tend"):
        if k in g:
            bad = np.nonzero(np.asarray(g[k])[:n] != o[k])[0]
            assert len(bad) == 0, (f"{label}: {k} differs on {len(bad)}/{n} records; first #{bad[0]}: "
                                   f"gpu {g[k][bad[0]]} oracle {o[k][bad[0]]}")
    hits = np.nonzero(o["hit"])[0]
    assert np.array_equal(np.asarray(g["hit_idx"], np.int64), hits), f"{label}: hit lists differ"
    if starts is not None:
        bad = np.nonzero(starts != o["start"][hits])[0]
        assert len(bad) == 0, (f"{label}: {len(bad)}/{len(hits)} starts differ; first record {hits[bad[0]]}: "
                               f"gpu {starts[bad[0]]} oracle {o['start'][hits[bad[0]]]}")
        assert np.array_equal(np.asarray(g["tend"])[hits] + 1, o["end"][hits]), f"{label}: match ends differ"
    return len(hits)


def _single(ctx, wl, q, algo, ends, gap_open, gap_ext, thr, label):
    qid = ctx.set_query(q, wl.kind, ScoringMatrix(wl.kind).values, algo, gap_open, gap_ext, ends,
                        _max_score(wl.kind, q), thr)
    sid = ctx.records_load(wl.records, wl.offsets)
    try:
        g = ctx.score_set(qid, sid)
        starts = ctx.match_starts(qid, sid, g["hit_idx"], g["tend"][g["hit_idx"]])
    finally:
        ctx.records_free(sid)
        ctx.free_query(qid)
    o = _oracle(wl, q, algo, ends, gap_open, gap_ext, thr)
    return _compare(g, o, label, starts)


FFTT = native.FREE_TARGET_START | native.FREE_TARGET_END


def test_line_search_workload(ctx):
    """ascii line search: 24-byte query, printable lines of 20-120 bytes, 1 % planted, thr 0.8."""
    wl = workloads.line_ascii(seed=0, n=20_000)
    nh = _single(ctx, wl, wl.queries[0], native.ALGO_SEMI_GLOBAL, FFTT, 3, 1, 0.8, "line")
    assert nh > 0


@pytest.mark.parametrize("thr", [0.8, 0.25])
def test_protein_workload(ctx, thr):
    """300-aa blosum62 query vs log-normal protein records, gap 10/1, semi-global FFTT and local."""
    wl = workloads.protein(seed=1, n=20_000, planted_frac=0.002)
    q = wl.queries[0]
    total = 0
    for algo, ends in ((native.ALGO_SEMI_GLOBAL, FFTT), (native.ALGO_LOCAL, 0)):
        total += _single(ctx, wl, q, algo, ends, 10, 1, thr, f"protein algo={algo} thr={thr}")
    if thr < 0.5:
        assert total > 0, "the lowered threshold should produce hits"


def test_batched_workload(ctx):
    """actgn reads of 100-300 nt with 0.5 % N, several queries of 50-1000 nt in one batched launch."""
    wl = workloads.nucleotide_multi(seed=2, nq=4, n=20_000)
    m = ScoringMatrix(wl.kind)
    qids = [ctx.set_query(q, wl.kind, m.values, native.ALGO_SEMI_GLOBAL, 3, 1, FFTT, _max_score(wl.kind, q), 0.8)
            for q in wl.queries]
    sid = ctx.records_load(wl.records, wl.offsets)
    try:
        r = ctx.score_multi(qids, sid)
        for i, q in enumerate(wl.queries):
            o = _oracle(wl, q, native.ALGO_SEMI_GLOBAL, FFTT, 3, 1, 0.8)
            g = {"score": r["score"][i], "qend": r["qend"][i], "tend": r["tend"][i], "hit_idx": r["hit_idx"][i]}
            _compare(g, o, f"batched query {i} (Q={len(q)})")
    finally:
        ctx.records_free(sid)
        for qid in qids:
            ctx.free_query(qid)
    # the reads carry no copies of the queries: plant 10 %-substituted copies
    # of the shortest query in 1 % of the reads long enough to hold one, so the
    # batched launch has hits to compact and start finding has starts to find
    q = min(wl.queries, key=len)
    rng = np.random.default_rng(22)
    lens = wl.lengths
    for i in rng.choice(np.nonzero(lens >= len(q))[0], wl.n // 100, replace=False):
        a, b = int(wl.offsets[i]), int(wl.offsets[i + 1])
        cp = q.copy()
        mut = rng.random(len(cp)) < 0.1
        cp[mut] = rng.integers(0, 4, int(mut.sum()), dtype=np.uint8)
        pos = int(rng.integers(0, b - a - len(cp) + 1))
        wl.records[a + pos:a + pos + len(cp)] = cp
    sid = ctx.records_load(wl.records, wl.offsets)
    qids = [ctx.set_query(q, wl.kind, m.values, native.ALGO_SEMI_GLOBAL, 3, 1, FFTT, _max_score(wl.kind, q), 0.8)]
    qids.append(ctx.set_query(wl.queries[0], wl.kind, m.values, native.ALGO_SEMI_GLOBAL, 3, 1, FFTT,
                              _max_score(wl.kind, wl.queries[0]), 0.8))
    try:
        r = ctx.score_multi(qids, sid)
        h = r["hit_idx"][0]
        starts = ctx.match_starts(qids[0], sid, h, r["tend"][0][h])
        o = _oracle(wl, q, native.ALGO_SEMI_GLOBAL, FFTT, 3, 1, 0.8)
        g = {"score": r["score"][0], "qend": r["qend"][0], "tend": r["tend"][0], "hit_idx": h}
        assert _compare(g, o, f"batched with planted copies (Q={len(q)})", starts) > 0
        o = _oracle(wl, wl.queries[0], native.ALGO_SEMI_GLOBAL, FFTT, 3, 1, 0.8)
        g = {"score": r["score"][1], "qend": r["qend"][1], "tend": r["tend"][1], "hit_idx": r["hit_idx"][1]}
        _compare(g, o, "batched beside it")
    finally:
        ctx.records_free(sid)
        for qid in qids:
            ctx.free_query(qid)


def test_long_target_workload(ctx):
    """1000-nt actgn0 query vs records of 10 kb-1 Mb (log-uniform) with planted 5 %-divergent copies."""
    wl = workloads.long_targets(seed=3, n=10, planted=5)
    nh = _single(ctx, wl, wl.queries[0], native.ALGO_SEMI_GLOBAL, FFTT, 3, 1, 0.8, "long")
    assert nh > 0
    assert ctx.last_windows() >= 0


def test_serving_workload(ctx):
    """Resident blosum62 set; a Poisson stream of queries of 20-2000 residues, local / semi-global mix."""
    wl = workloads.serving_records(seed=4, total_bytes=6 << 20)
    qs = workloads.serving_queries(count=3, rate=50.0)
    m = ScoringMatrix(wl.kind)
    # plant 15 %-substituted copies of each query in a few records at least as
    # long as the query (the longest records where there are too few) so every
    # query has hits
    rng = np.random.default_rng(44)
    lens = wl.lengths
    for _, _, q in qs:
        cand = np.nonzero(lens >= len(q))[0]
        if len(cand) < 6:
            cand = np.argsort(lens)[-6:]
        for i in rng.choice(cand, 6, replace=False):
            a, b = int(wl.offsets[i]), int(wl.offsets[i + 1])
            cp = q[: b - a].copy()
            mut = rng.random(len(cp)) < 0.15
            cp[mut] = rng.integers(0, 20, int(mut.sum()), dtype=np.uint8)
            pos = int(rng.integers(0, b - a - len(cp) + 1))
            wl.records[a + pos:a + pos + len(cp)] = cp
    sid = ctx.records_load(wl.records, wl.offsets)
    ids, meta = [], []
    for _, algo_name, q in qs:
        algo = native.ALGO_LOCAL if algo_name == "striped-local" else native.ALGO_SEMI_GLOBAL
        ends = 0 if algo == native.ALGO_LOCAL else FFTT
        # threshold 0.3: random records against random queries give no hits at 0.8
        ids.append(ctx.set_query(q, wl.kind, m.values, algo, 10, 1, ends, _max_score(wl.kind, q), 0.3))
        meta.append((q, algo, ends))
    try:
        ctx.serve_start(sid, max_active=8, chunks=4)
        try:
            tickets = [ctx.submit(qid) for qid in ids]
            results = []
            for t in tickets:
                r = None
                while r is None:
                    r = ctx.poll(t, wait_ms=200)
                results.append(r)
        finally:
            ctx.serve_stop()
        for (q, algo, ends), r in zip(meta, results):
            o = _oracle(wl, q, algo, ends, 10, 1, 0.3)
            hits = np.nonzero(o["hit"])[0]
            label = f"serving algo={algo} Q={len(q)}"
            assert np.array_equal(np.asarray(r["hit_idx"], np.int64), hits), f"{label}: hit lists differ"
            for k in ("score", "qend", "tend"):
                assert np.array_equal(r[k], o[k][hits]), f"{label}: {k} of the hits differs"
        assert sum(len(r["hit_idx"]) for r in results) > 0
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)

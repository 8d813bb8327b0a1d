"""The serving loop: continuous batching against a resident record set.

Queries submitted while others run are admitted at the next step and share
the device with them.  Each query's result -- its hit list with the score and
end coordinates of every hit -- must be exactly what the query gets alone
(ish_gpu_score_set), whatever mix it ran in.
"""
import threading

import numpy as np
import pytest

from ish_gb300 import native
from ish_gb300.scoring import BLOSUM62, ScoringMatrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    # every query takes the server's full chunk count: these sets are small,
    # and the adaptive step size would score most queries in one step
    c.set_option(native.OPT_SERVE_STEP_CELLS, 0)
    yield c
    c.close()


def protein_set(rng, n, queries, plant=0.03):
    recs = []
    for _ in range(n):
        L = int(np.clip(rng.lognormal(np.log(350), 0.6), 30, 3000))
        r = rng.integers(0, 20, L, dtype=np.uint8)
        if rng.random() < plant:
            q = queries[int(rng.integers(0, len(queries)))]
            if len(q) <= L:
                pos = int(rng.integers(0, L - len(q) + 1))
                cp = q.copy()
                mut = rng.random(len(cp)) < 0.15
                cp[mut] = rng.integers(0, 20, int(mut.sum()), dtype=np.uint8)
                r[pos:pos + len(cp)] = cp
        recs.append(r)
    recs.append(np.zeros(0, np.uint8))  # an empty record
    return native.pack_records(recs)


def make_queries(ctx, rng, lens, thr=0.4):
    m = ScoringMatrix(BLOSUM62)
    seqs, ids = [], []
    for i, L in enumerate(lens):
        q = rng.integers(0, 20, L, dtype=np.uint8)
        algo = native.ALGO_LOCAL if i % 2 else native.ALGO_SEMI_GLOBAL
        ends = 0 if algo == native.ALGO_LOCAL else (12 if i % 4 == 0 else 15)
        ids.append(ctx.set_query(q, BLOSUM62, m.values, algo, 10, 1, ends, int(m.values[q, q].sum()), thr))
        seqs.append(q)
    return seqs, ids


def alone(ctx, qid, sid):
    r = ctx.score_set(qid, sid)
    h = r["hit_idx"]
    return {"hit_idx": h, "score": r["score"][h], "qend": r["qend"][h], "tend": r["tend"][h]}


def same(a, b, label):
    for k in ("hit_idx", "score", "qend", "tend"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), f"{label}: {k} differs"


def wait(ctx, ticket, timeout_s=120):
    for _ in range(int(timeout_s * 10)):
        r = ctx.poll(ticket, wait_ms=100)
        if r is not None:
            return r
    raise AssertionError(f"ticket {ticket} did not finish in {timeout_s} s")


def test_serving_results_equal_alone_under_concurrency(ctx):
    rng = np.random.default_rng(51)
    lens = [20, 45, 90, 150, 200, 260, 300, 333, 410, 500, 640, 777]
    seqs, ids = make_queries(ctx, rng, lens)
    buf, off = protein_set(rng, 6000, seqs)
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids]
        assert sum(len(e["hit_idx"]) for e in expect) > 0
        ctx.serve_start(sid, max_active=16, mem_budget=0, chunks=8)
        try:
            # three client threads submit and poll concurrently
            tickets = {}
            results = {}
            lock = threading.Lock()

            def client(part):
                mine = [(i, ctx.submit(ids[i])) for i in part]
                with lock:
                    tickets.update(dict(mine))
                for i, t in mine:
                    r = wait(ctx, t)
                    with lock:
                        results[i] = r

            th = [threading.Thread(target=client, args=(list(range(k, len(ids), 3)),)) for k in range(3)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            assert len(results) == len(ids)
            for i in range(len(ids)):
                same(results[i], expect[i], f"query {i} (Q={lens[i]})")
                assert results[i]["latency_ms"] > 0
            # a second wave with duplicates, submitted while the first runs
            t1 = [ctx.submit(ids[i]) for i in (3, 3, 7, 0)]
            t2 = [ctx.submit(ids[i]) for i in (11, 3)]
            for t, i in zip(t1 + t2, (3, 3, 7, 0, 11, 3)):
                same(wait(ctx, t), expect[i], f"repeat of query {i}")
            st = ctx.serve_stats()
            assert st["completed"] == len(ids) + 6
            assert st["max_active"] >= 2, st  # requests shared steps
            assert st["cells"] > 0 and st["device_ms"] > 0
        finally:
            ctx.serve_stop()
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_serving_memory_budget_admits_one_at_a_time(ctx):
    rng = np.random.default_rng(52)
    seqs, ids = make_queries(ctx, rng, [60, 120, 240])
    buf, off = protein_set(rng, 2000, seqs)
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids]
        ctx.serve_start(sid, max_active=8, mem_budget=1, chunks=4)  # room for one request's outputs
        try:
            ts = [ctx.submit(q) for q in ids]
            for t, e, L in zip(ts, expect, (60, 120, 240)):
                same(wait(ctx, t), e, f"Q={L}")
            assert ctx.serve_stats()["max_active"] == 1
        finally:
            ctx.serve_stop()
    finally:
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_serving_errors_stay_with_their_request(ctx):
    rng = np.random.default_rng(53)
    seqs, ids = make_queries(ctx, rng, [80, 0])
    # a nucleotide query (5-letter alphabet) against protein records (codes up
    # to 19) cannot run: its request fails alone
    dna = ScoringMatrix(1)
    qd = rng.integers(0, 5, 50, dtype=np.uint8)
    bad = ctx.set_query(qd, 1, dna.values, native.ALGO_SEMI_GLOBAL, 3, 1, 12, int(dna.values[qd, qd].sum()), 0.5)
    buf, off = protein_set(rng, 1500, seqs[:1])
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids]
        ctx.serve_start(sid, max_active=4, chunks=3)
        try:
            with pytest.raises(native.IshGpuError):
                ctx.records_free(sid)  # in use by the serving loop
            with pytest.raises(native.IshGpuError):
                ctx.set_option(native.OPT_WAVE_LEAN, 1)  # the serving thread reads the options
            tb = ctx.submit(bad)
            t0, t1 = ctx.submit(ids[0]), ctx.submit(ids[1])
            with pytest.raises(native.IshGpuError) as ei:
                wait(ctx, tb)
            assert ei.value.code == native.EINVAL
            same(wait(ctx, t0), expect[0], "good query next to a failing one")
            same(wait(ctx, t1), expect[1], "empty query")
            with pytest.raises(native.IshGpuError):
                ctx.poll(t0)  # delivered once
        finally:
            ctx.serve_stop()
    finally:
        ctx.records_free(sid)
        for qid in ids + [bad]:
            ctx.free_query(qid)


def test_serving_exact_kernel_requests(ctx):
    # gap_open == gap_extend puts a query outside the wavefront kernels'
    # regime: the serving loop scores its chunks with the lane-exact kernels,
    # next to wavefront requests, and results still equal the query alone
    rng = np.random.default_rng(54)
    m = ScoringMatrix(BLOSUM62)
    seqs, ids = make_queries(ctx, rng, [70, 140])
    q = rng.integers(0, 20, 90, dtype=np.uint8)
    ex = [ctx.set_query(q, BLOSUM62, m.values, algo, 2, 2, ends, int(m.values[q, q].sum()), 0.3)
          for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_LOCAL, 0))]
    buf, off = protein_set(rng, 1200, seqs + [q])
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids + ex]
        ctx.serve_start(sid, max_active=8, chunks=3)
        try:
            ts = [ctx.submit(qid) for qid in ids + ex]
            for t, e, i in zip(ts, expect, range(4)):
                same(wait(ctx, t), e, f"request {i}")
        finally:
            ctx.serve_stop()
    finally:
        ctx.records_free(sid)
        for qid in ids + ex:
            ctx.free_query(qid)


def test_serving_windows_long_records(ctx):
    # a served set with a few 40-60 kb records: requests whose window fold is
    # exact score a shared window view (a later request with a larger overlap
    # gets a new one); every result equals the query alone (single-query
    # scoring windows the set itself) and the unwindowed loop
    rng = np.random.default_rng(57)
    m = ScoringMatrix(BLOSUM62)
    specs = [(80, native.ALGO_SEMI_GLOBAL, 12), (60, native.ALGO_LOCAL, 0), (120, native.ALGO_SEMI_GLOBAL, 13),
             (200, native.ALGO_LOCAL, 0), (150, native.ALGO_SEMI_GLOBAL, 12)]
    seqs, ids = [], []
    for L, algo, ends in specs:
        q = rng.integers(0, 20, L, dtype=np.uint8)
        ids.append(ctx.set_query(q, BLOSUM62, m.values, algo, 10, 1, ends, int(m.values[q, q].sum()), 0.4))
        seqs.append(q)
    buf, off = protein_set(rng, 1500, seqs, plant=0.05)
    recs = [buf[int(off[i]):int(off[i + 1])] for i in range(len(off) - 1)]
    for L in (40_000, 52_000, 60_000):
        r = rng.integers(0, 20, L, dtype=np.uint8)
        for q in seqs:
            pos = int(rng.integers(0, L - len(q)))
            r[pos:pos + len(q)] = q
        recs.insert(int(rng.integers(0, len(recs))), r)
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids]
        for windows in (1, 0):
            ctx.set_option(native.OPT_WINDOWS, windows)
            ctx.serve_start(sid, max_active=8, mem_budget=0, chunks=4)
            try:
                tickets = [ctx.submit(qid) for qid in ids]
                for i, t in enumerate(tickets):
                    same(wait(ctx, t), expect[i], f"query {i} (windows {windows})")
                # again, one at a time (each admitted alone)
                for i, qid in enumerate(ids):
                    same(wait(ctx, ctx.submit(qid)), expect[i], f"query {i} alone (windows {windows})")
            finally:
                ctx.serve_stop()
    finally:
        ctx.set_option(native.OPT_WINDOWS, 1)
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)


def test_serving_adaptive_steps(ctx):
    # the default step size: queries whose work is small (here at most 8e9
    # cells) take one step instead of the server's 8 chunks; results are
    # unchanged
    rng = np.random.default_rng(71)
    seqs, ids = make_queries(ctx, rng, [30, 120, 400, 900])
    buf, off = protein_set(rng, 20000, seqs)
    sid = ctx.records_load(buf, off)
    try:
        expect = [alone(ctx, qid, sid) for qid in ids]
        for cells in (1.25e11, 0):  # 0: every query takes all 8 chunks
            ctx.set_option(native.OPT_SERVE_STEP_CELLS, int(cells))
            ctx.serve_start(sid, max_active=8, chunks=8)
            try:
                tickets = [ctx.submit(qid) for qid in ids]
                for i, t in enumerate(tickets):
                    same(wait(ctx, t), expect[i], f"query {i} (step cells {cells:g})")
                steps = ctx.serve_stats()["steps"]
            finally:
                ctx.serve_stop()
            if cells:
                assert steps <= 4, steps  # one step per query at most (shared when they overlap)
            else:
                assert steps >= 8, steps
    finally:
        ctx.set_option(native.OPT_SERVE_STEP_CELLS, 0)
        ctx.records_free(sid)
        for qid in ids:
            ctx.free_query(qid)

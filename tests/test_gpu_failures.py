"""Failure detection without a GPU fault.

Two hooks make a failure happen on purpose, and each test checks that the call
reports it as a status and that the same context then scores bit-exactly:

* ISH_OPT_STEP_BUDGET caps every warp of a wavefront or batched launch at a few
  pipeline steps.  The bound every launch already carries runs out, the kernel
  stops and returns, and the call fails with ISH_ETIMEDOUT -- the device-side
  bound made to run out, not a hang, trap or bad address.
* ISH_OPT_FAULT_ALLOC makes the next device allocation fail on the host, as if
  device memory were exhausted; the call fails with ISH_ENOMEM.
"""
import os

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import BLOSUM62, ScoringMatrix

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4
FFTT = native.FREE_TARGET_START | native.FREE_TARGET_END


@pytest.fixture()
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.set_option(native.OPT_FAULT_ALLOC, -1)
    c.close()


def protein(rng, n, q):
    recs = []
    for i in range(n):
        L = int(np.clip(rng.lognormal(np.log(350), 0.6), 30, 3000))
        r = rng.integers(0, 20, L, dtype=np.uint8)
        if i % 25 == 0 and L >= len(q):
            p = int(rng.integers(0, L - len(q) + 1))
            cp = q.copy()
            mut = rng.random(len(cp)) < 0.2
            cp[mut] = rng.integers(0, 20, int(mut.sum()), dtype=np.uint8)
            r[p:p + len(cp)] = cp
        recs.append(r)
    return native.pack_records(recs)


def set_query(ctx, q, algo, thr=0.4):
    m = ScoringMatrix(BLOSUM62)
    return ctx.set_query(q, BLOSUM62, m.values, algo, 10, 1, FFTT if algo == native.ALGO_SEMI_GLOBAL else 0,
                         int(m.values[q, q].sum()), thr)


def oracle(buf, off, q, algo, thr=0.4):
    m = ScoringMatrix(BLOSUM62)
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, BLOSUM62, q,
                   int(m.values[q, q].sum()), thr, gap_open=10, gap_extend=1,
                   ends=FFTT if algo == native.ALGO_SEMI_GLOBAL else 0)
    return om.batch(buf, off, threads=THREADS)


def same(g, o, label):
    for k in ("score", "qend", "tend"):
        assert np.array_equal(g[k], o[k]), f"{label}: {k} differs from the oracle"
    assert np.array_equal(np.asarray(g["hit_idx"], np.int64), np.nonzero(o["hit"])[0]), f"{label}: hits differ"


def expect(code, fn, *a, **kw):
    with pytest.raises(native.IshGpuError) as e:
        fn(*a, **kw)
    assert e.value.code == code, str(e.value)


@pytest.mark.parametrize("algo", [native.ALGO_SEMI_GLOBAL, native.ALGO_LOCAL])
def test_step_budget_runs_out_then_context_is_usable(ctx, algo):
    rng = np.random.default_rng(5 + algo)
    q = rng.integers(0, 20, 300, dtype=np.uint8)
    buf, off = protein(rng, 3000, q)
    qid = set_query(ctx, q, algo)
    sid = ctx.records_load(buf, off)
    ctx.set_option(native.OPT_STEP_BUDGET, 16)
    expect(native.ETIMEDOUT, ctx.score_set, qid, sid)
    expect(native.ETIMEDOUT, ctx.score, qid, buf, off)
    ctx.set_option(native.OPT_STEP_BUDGET, 0)
    o = oracle(buf, off, q, algo)
    same(ctx.score_set(qid, sid), o, "resident set after the timeout")
    same(ctx.score(qid, buf, off), o, "one-shot call after the timeout")


def test_step_budget_batched_launch(ctx):
    rng = np.random.default_rng(9)
    qs = [rng.integers(0, 20, L, dtype=np.uint8) for L in (60, 300, 700)]
    buf, off = protein(rng, 2000, qs[1])
    qids = [set_query(ctx, q, native.ALGO_SEMI_GLOBAL if i % 2 == 0 else native.ALGO_LOCAL) for i, q in enumerate(qs)]
    sid = ctx.records_load(buf, off)
    ctx.set_option(native.OPT_STEP_BUDGET, 16)
    expect(native.ETIMEDOUT, ctx.score_multi, qids, sid)
    ctx.set_option(native.OPT_STEP_BUDGET, 0)
    r = ctx.score_multi(qids, sid)
    for i, q in enumerate(qs):
        o = oracle(buf, off, q, native.ALGO_SEMI_GLOBAL if i % 2 == 0 else native.ALGO_LOCAL)
        same({"score": r["score"][i], "qend": r["qend"][i], "tend": r["tend"][i], "hit_idx": r["hit_idx"][i]}, o,
             f"batched query {i}")


def test_step_budget_serving_loop(ctx):
    rng = np.random.default_rng(13)
    q = rng.integers(0, 20, 250, dtype=np.uint8)
    buf, off = protein(rng, 3000, q)
    qid = set_query(ctx, q, native.ALGO_LOCAL)
    sid = ctx.records_load(buf, off)
    ctx.set_option(native.OPT_STEP_BUDGET, 16)
    ctx.serve_start(sid, max_active=4, chunks=2)
    try:
        t = ctx.submit(qid)
        with pytest.raises(native.IshGpuError) as e:
            while ctx.poll(t, wait_ms=200) is None:
                pass
        assert e.value.code == native.ETIMEDOUT, str(e.value)
    finally:
        ctx.serve_stop()
    ctx.set_option(native.OPT_STEP_BUDGET, 0)
    ctx.serve_start(sid, max_active=4, chunks=2)
    try:
        t = ctx.submit(qid)
        r = None
        while r is None:
            r = ctx.poll(t, wait_ms=200)
    finally:
        ctx.serve_stop()
    o = oracle(buf, off, q, native.ALGO_LOCAL)
    hits = np.nonzero(o["hit"])[0]
    assert len(hits) > 0
    assert np.array_equal(np.asarray(r["hit_idx"], np.int64), hits)
    for k in ("score", "qend", "tend"):
        assert np.array_equal(r[k], o[k][hits])


def test_injected_allocation_failure(ctx):
    rng = np.random.default_rng(17)
    q = rng.integers(0, 20, 200, dtype=np.uint8)
    small_buf, small_off = protein(rng, 200, q)
    buf, off = protein(rng, 4000, q)
    qid = set_query(ctx, q, native.ALGO_SEMI_GLOBAL)
    ctx.score(qid, small_buf, small_off)  # warm: everything a small call needs is allocated
    # a larger set needs larger buffers: the first allocation fails
    ctx.set_option(native.OPT_FAULT_ALLOC, 0)
    expect(native.ENOMEM, ctx.records_load, buf, off)
    sid = ctx.records_load(buf, off)  # the fault fired once and disarmed
    o = oracle(buf, off, q, native.ALGO_SEMI_GLOBAL)
    same(ctx.score_set(qid, sid), o, "set loaded after the failed load")
    # one-shot scoring of a larger batch: its output buffers grow
    buf2, off2 = protein(rng, 9000, q)
    ctx.set_option(native.OPT_FAULT_ALLOC, 0)
    expect(native.ENOMEM, ctx.score, qid, buf2, off2)
    same(ctx.score(qid, buf2, off2), oracle(buf2, off2, q, native.ALGO_SEMI_GLOBAL), "one-shot call after ENOMEM")
    # the serving loop's own buffers
    ctx.set_option(native.OPT_FAULT_ALLOC, 0)
    expect(native.ENOMEM, ctx.serve_start, sid, 4, 0, 2)
    ctx.serve_start(sid, max_active=4, chunks=2)
    try:
        t = ctx.submit(qid)
        r = None
        while r is None:
            r = ctx.poll(t, wait_ms=200)
    finally:
        ctx.serve_stop()
    hits = np.nonzero(o["hit"])[0]
    assert np.array_equal(np.asarray(r["hit_idx"], np.int64), hits)
    # a later allocation in the countdown: the second one fails
    ctx.set_option(native.OPT_FAULT_ALLOC, 1)
    with pytest.raises(native.IshGpuError) as e:
        for _ in range(4):
            s2 = ctx.records_load(*protein(rng, 20000, q))
            ctx.records_free(s2)
    assert e.value.code == native.ENOMEM
    ctx.set_option(native.OPT_FAULT_ALLOC, -1)
    same(ctx.score_set(qid, sid), o, "resident set after the second fault")


def test_allocation_failure_at_every_step_of_a_load(ctx):
    """A load that fails at any one of its device allocations -- before the
    packing kernels start, or after the first of them have run and touched the
    shared length histogram -- leaves the context able to load and score: the
    next load's results equal the oracle's.  Each attempt is larger than the
    one before, so its buffers grow and allocate; the countdown picks which
    allocation fails, and the synchronous and the asynchronous load alternate."""
    rng = np.random.default_rng(23)
    q = rng.integers(0, 20, 120, dtype=np.uint8)
    qid = set_query(ctx, q, native.ALGO_SEMI_GLOBAL)
    good_buf, good_off = protein(rng, 300, q)
    o = oracle(good_buf, good_off, q, native.ALGO_SEMI_GLOBAL)
    size, failures = 600, 0
    for k in range(8):
        size = int(size * 1.5)
        buf, off = protein(rng, size, q)
        load = ctx.records_load if k % 2 == 0 else ctx.records_load_async
        ctx.set_option(native.OPT_FAULT_ALLOC, k)
        try:
            sid = load(buf, off)
            ctx.records_info(sid)  # an asynchronous load completes here
            ctx.records_free(sid)
        except native.IshGpuError as e:
            assert e.code == native.ENOMEM, str(e)
            failures += 1
        ctx.set_option(native.OPT_FAULT_ALLOC, -1)
        sid = ctx.records_load(good_buf, good_off)
        same(ctx.score_set(qid, sid), o, f"load after a fault at allocation {k}")
        ctx.records_free(sid)
    assert failures >= 3

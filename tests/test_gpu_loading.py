"""Records prepared on the device: raw bytes encoded while packing
(ish_gpu_records_load_raw) and text split into line records
(ish_gpu_records_load_lines).  Both must give exactly the set the host path
gives -- records encoded and split as ish's runners do -- and therefore
identical scores."""
import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import ScoringMatrix
from searcher_fixtures import kseq_lines

pytestmark = pytest.mark.gpu

KINDS = [O.ASCII, O.ACTGN, O.ACTGN0, O.BLOSUM62]


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.close()


def query_for(ctx, kind, rng, qlen=30, algo=native.ALGO_SEMI_GLOBAL, ends=12):
    m = ScoringMatrix(kind)
    q = m.encode(rng.choice(np.frombuffer(b"ACGTNacgtnRDEQHKLMxyz*#", np.uint8), qlen).tobytes())
    return ctx.set_query(q, kind, m.values, algo, 3, 1, ends, int(m.values[q, q].sum()), 0.3), m


def same_results(ctx, qid, a, b):
    ra, rb = ctx.score_set(qid, a), ctx.score_set(qid, b)
    for k in ("score", "qend", "tend", "hit"):
        assert np.array_equal(ra[k], rb[k]), k
    assert np.array_equal(ra["hit_idx"], rb["hit_idx"])


def random_text(rng, nlines):
    parts = []
    for i in range(nlines):
        L = int(rng.integers(0, 90))
        line = rng.choice(np.frombuffer(b"ACGTacgtNRDEQ \t*xyz\x00", np.uint8), L).tobytes()
        end = [b"\n", b"\r\n", b"\n", b"\r\r\n"][int(rng.integers(0, 4))]
        if rng.random() < 0.05:
            line = b"\r"  # a lone carriage return is kept
        parts.append(line + end)
    text = b"".join(parts)
    if rng.random() < 0.5:
        text += b"tail without newline\r"
    return text


@pytest.mark.parametrize("kind", KINDS)
def test_lines_split_and_encoded_on_device(ctx, kind):
    rng = np.random.default_rng(40 + kind)
    for trial in range(4):
        text = random_text(rng, int(rng.integers(1, 3000)))
        lines = kseq_lines(text)
        m = ScoringMatrix(kind)
        enc = [m.encode(l) for l in lines]
        buf, off = native.pack_records(enc)
        sid_d, n = ctx.records_load_lines(text, kind)
        sid_h = ctx.records_load(buf, off)
        try:
            assert n == len(lines)
            assert ctx.records_info(sid_d) == (len(lines), int(off[-1]))
            qid, _ = query_for(ctx, kind, rng)
            same_results(ctx, qid, sid_d, sid_h)
            ctx.free_query(qid)
        finally:
            ctx.records_free(sid_d)
            ctx.records_free(sid_h)


@pytest.mark.parametrize("kind", KINDS)
def test_raw_bytes_encoded_on_device(ctx, kind):
    rng = np.random.default_rng(60 + kind)
    recs = [rng.integers(0, 256, int(rng.integers(0, 300)), dtype=np.uint8) for _ in range(2000)]
    raw, off = native.pack_records(recs)
    m = ScoringMatrix(kind)
    enc = m.encode(raw)
    sid_d = ctx.records_load_raw(raw, off, kind)
    sid_h = ctx.records_load(enc, off)
    try:
        for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_LOCAL, 0)):
            qid, _ = query_for(ctx, kind, rng, 40, algo, ends)
            same_results(ctx, qid, sid_d, sid_h)
            ctx.free_query(qid)
    finally:
        ctx.records_free(sid_d)
        ctx.records_free(sid_h)


def test_line_edge_cases(ctx):
    for text in (b"", b"\n", b"\n\n", b"a", b"a\n", b"\r\n", b"\r", b"ab\r", b"x\r\r\n\ny"):
        lines = kseq_lines(text)
        sid, n = ctx.records_load_lines(text, O.ASCII)
        try:
            assert n == len(lines), text
            assert ctx.records_info(sid) == (len(lines), sum(len(l) for l in lines)), text
        finally:
            ctx.records_free(sid)


def test_lines_against_oracle(ctx):
    # end to end: text in, hits out, compared with the oracle on host-split lines
    rng = np.random.default_rng(77)
    pat = b"GATTACAGATTACA"
    lines = [bytes(rng.choice(list(b"ACGT"), int(rng.integers(5, 120)))) for _ in range(3000)]
    lines = [l[:7] + pat + l[7:] if i % 9 == 0 else l for i, l in enumerate(lines)]
    text = b"\r\n".join(lines) + b"\n"
    om = O.Matcher.from_ascii(O.SEMI_GLOBAL, O.ACTGN, pat, 0.8, ends=O.TS | O.TE)
    m = ScoringMatrix(O.ACTGN)
    q, mx = m.encode_and_score(pat)
    qid = ctx.set_query(q, O.ACTGN, m.values, native.ALGO_SEMI_GLOBAL, 3, 1, 12, mx, 0.8)
    sid, n = ctx.records_load_lines(text, O.ACTGN)
    try:
        r = ctx.score_set(qid, sid)
        want = [i for i, l in enumerate(kseq_lines(text)) if om.first_match(m.encode(l)) is not None]
        assert list(r["hit_idx"]) == want and len(want) >= 300
    finally:
        ctx.records_free(sid)
        ctx.free_query(qid)


def test_freed_set_buffers_are_reused_exactly(ctx):
    # records_free keeps a freed set's device buffers for the next load: sets
    # of other sizes loaded into them score exactly like a set loaded fresh
    rng = np.random.default_rng(47)
    qid, m = query_for(ctx, O.BLOSUM62, rng, qlen=40)

    def make(n, lo, hi):
        recs = [rng.integers(0, 20, int(rng.integers(lo, hi)), dtype=np.uint8) for _ in range(n)]
        return native.pack_records(recs)

    sets = [make(3000, 50, 400), make(500, 1, 40), make(8000, 100, 900), make(2, 0, 3)]
    keep = [ctx.records_load(b, o) for b, o in sets]  # fresh buffers: the expected results
    expect = [ctx.score_set(qid, s) for s in keep]
    for s in keep:
        ctx.records_free(s)
    try:
        for order in ([0, 1, 2, 3], [2, 0, 3, 1], [1, 1, 2, 2, 0]):
            for i in order:
                sid = ctx.records_load(*sets[i])
                got = ctx.score_set(qid, sid)
                ctx.records_free(sid)
                for k in ("score", "qend", "tend", "hit", "hit_idx"):
                    assert np.array_equal(got[k], expect[i][k]), (order, i, k)
        # two sets alive at once take different buffers
        a, b = ctx.records_load(*sets[0]), ctx.records_load(*sets[2])
        ra, rb = ctx.score_set(qid, a), ctx.score_set(qid, b)
        assert np.array_equal(ra["score"], expect[0]["score"]) and np.array_equal(rb["score"], expect[2]["score"])
        ctx.records_free(a)
        ctx.records_free(b)
    finally:
        ctx.free_query(qid)


def test_async_load_equals_sync_and_overlaps_scoring(ctx):
    # records_load_async: the set's upload and packing run on the load stream;
    # scoring another set meanwhile, then using the new set, gives exactly
    # what a synchronous load gives; a pending set may also be freed unused,
    # replaced by another load, or left for close
    rng = np.random.default_rng(61)
    m = ScoringMatrix(O.BLOSUM62)
    q = rng.integers(0, 20, 150, dtype=np.uint8)
    qid = ctx.set_query(q, O.BLOSUM62, m.values, native.ALGO_SEMI_GLOBAL, 10, 1,
                        native.FREE_TARGET_START | native.FREE_TARGET_END, int(m.values[q, q].sum()), 0.5)
    batches = []
    for b in range(4):
        recs = [rng.integers(0, 20, int(rng.integers(0, 900)), dtype=np.uint8) for _ in range(3000 + 500 * b)]
        for r in recs[::50]:
            if len(r) >= len(q) + 3:
                r[3:3 + len(q)] = q
        batches.append(native.pack_records(recs))
    want = []
    for buf, off in batches:
        sid = ctx.records_load(buf, off)
        want.append(ctx.score_set(qid, sid))
        ctx.records_free(sid)
    # pipelined: load b + 1 asynchronously, then score b
    sid = ctx.records_load_async(*batches[0])
    for b in range(4):
        nxt = ctx.records_load_async(*batches[b + 1]) if b + 1 < 4 else None
        got = ctx.score_set(qid, sid)
        for k in ("score", "qend", "tend", "hit", "hit_idx"):
            assert np.array_equal(got[k], want[b][k]), (b, k)
        assert ctx.records_info(sid)[0] == len(batches[b][1]) - 1
        ctx.records_free(sid)
        sid = nxt
    # a pending set freed without use, then one replaced by a synchronous load
    sid = ctx.records_load_async(*batches[1])
    ctx.records_free(sid)
    sid = ctx.records_load_async(*batches[2])
    sid2 = ctx.records_load(*batches[3])
    for s, b in ((sid, 2), (sid2, 3)):
        got = ctx.score_set(qid, s)
        assert np.array_equal(got["score"], want[b]["score"]) and np.array_equal(got["hit_idx"], want[b]["hit_idx"])
        ctx.records_free(s)
    # the one-shot call after an asynchronous load
    sid = ctx.records_load_async(*batches[0])
    one = ctx.score(qid, *batches[1])
    assert np.array_equal(one["score"], want[1]["score"])
    assert np.array_equal(ctx.score_set(qid, sid)["score"], want[0]["score"])
    ctx.records_free(sid)
    ctx.free_query(qid)


def test_async_load_pending_at_close():
    # a context closed with its asynchronous load still in flight
    rng = np.random.default_rng(62)
    buf, off = native.pack_records([rng.integers(0, 20, 500, dtype=np.uint8) for _ in range(2000)])
    c = native.Context(0)
    c.records_load_async(buf, off)
    c.close()

"""Parity of the CUDA engine with the CPU oracle (bit-exact integers).

Every case scores the same seeded records through libish_gpu.so (C ABI) and
through the oracle's restatement of ish's striped matchers, and requires
identical scores, end coordinates and hit flags for every record.
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
ALL_ENDS = list(range(16))


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.close()


def random_records(rng, alphabet, n, lmin, lmax, query=None, plant_frac=0.2, sub=0.1):
    recs = []
    for _ in range(n):
        L = int(rng.integers(lmin, lmax + 1))
        r = rng.integers(0, alphabet, L, dtype=np.uint8)
        if query is not None and len(query) and L >= len(query) and rng.random() < plant_frac:
            pos = int(rng.integers(0, L - len(query) + 1))
            cp = query.copy()
            mut = rng.random(len(cp)) < sub
            cp[mut] = rng.integers(0, alphabet, int(mut.sum()), dtype=np.uint8)
            r[pos:pos + len(cp)] = cp
        recs.append(r)
    return recs


def run_both(ctx, algo, kind, q, recs, gap_open, gap_ext, ends, thr=0.5, kernel=native.KERNEL_AUTO):
    m = ScoringMatrix(kind)
    max_score = int(m.values[q, q].astype(np.int64).sum()) if len(q) else 0
    buf, off = native.pack_records(recs)
    ctx.set_option(native.OPT_KERNEL, kernel)
    qid = ctx.set_query(q, kind, m.values, algo, gap_open, gap_ext, ends, max_score, thr)
    try:
        g = ctx.score(qid, buf, off)
    finally:
        ctx.free_query(qid)
        ctx.set_option(native.OPT_KERNEL, native.KERNEL_AUTO)
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, kind, q, max_score, thr,
                   gap_open=gap_open, gap_extend=gap_ext, ends=ends)
    o = om.batch(buf, off, threads=THREADS)
    return g, o


def assert_same(g, o, label=""):
    n = len(o["score"])
    for k_g, k_o in (("score", "score"), ("qend", "qend"), ("tend", "tend"), ("hit", "hit")):
        bad = np.nonzero(g[k_g][:n] != o[k_o][:n])[0]
        if len(bad):
            i = bad[0]
            raise AssertionError(
                f"{label}: {k_g} differs on {len(bad)}/{n} records; first #{i}: gpu "
                f"({g['score'][i]}, {g['qend'][i]}, {g['tend'][i]}, {g['hit'][i]}) oracle "
                f"({o['score'][i]}, {o['qend'][i]}, {o['tend'][i]}, {o['hit'][i]})")
    assert (g["hit_idx"] == np.nonzero(o["hit"])[0]).all(), label


QLENS = [1, 2, 5, 17, 24, 33, 64, 100, 255, 300, 511, 800]


@pytest.mark.parametrize("qlen", QLENS)
@pytest.mark.parametrize("kind", [O.ACTGN, O.BLOSUM62])
def test_semi_global_random(ctx, qlen, kind):
    rng = np.random.default_rng(1000 + qlen + 7 * kind)
    alpha = 5 if kind == O.ACTGN else 20
    q = rng.integers(0, alpha, qlen, dtype=np.uint8)
    recs = random_records(rng, alpha, 120, 0, 2 * qlen + 40, q)
    for ends in ALL_ENDS:
        g, o = run_both(ctx, native.ALGO_SEMI_GLOBAL, kind, q, recs, 10 if kind == O.BLOSUM62 else 3, 1, ends)
        assert_same(g, o, f"SG kind={kind} Q={qlen} ends={ends}")


@pytest.mark.parametrize("qlen", QLENS)
@pytest.mark.parametrize("kind", [O.ACTGN, O.ACTGN0, O.BLOSUM62])
def test_local_random(ctx, qlen, kind):
    rng = np.random.default_rng(2000 + qlen + 7 * kind)
    alpha = 5 if kind in (O.ACTGN, O.ACTGN0) else 24
    q = rng.integers(0, alpha, qlen, dtype=np.uint8)
    recs = random_records(rng, alpha, 150, 0, 2 * qlen + 40, q)
    g, o = run_both(ctx, native.ALGO_LOCAL, kind, q, recs, 10 if kind == O.BLOSUM62 else 3, 1, 0)
    assert_same(g, o, f"SW kind={kind} Q={qlen}")


@pytest.mark.parametrize("algo", [native.ALGO_SEMI_GLOBAL, native.ALGO_LOCAL])
def test_ascii_small_alphabet_ties(ctx, algo):
    # four distinct bytes: many equal scores, exercises every tie rule
    rng = np.random.default_rng(7)
    for qlen in (3, 24, 70):
        q = rng.integers(65, 69, qlen, dtype=np.uint8)
        recs = [rng.integers(65, 69, int(rng.integers(0, 150)), dtype=np.uint8) for _ in range(200)]
        for ends in (ALL_ENDS if algo == native.ALGO_SEMI_GLOBAL else [0]):
            g, o = run_both(ctx, algo, O.ASCII, q, recs, 3, 1, ends, thr=0.3)
            assert_same(g, o, f"ascii algo={algo} Q={qlen} ends={ends}")


@pytest.mark.parametrize("G", [1, 2, 4, 8, 16, 32])
def test_forced_group_shapes(ctx, G):
    rng = np.random.default_rng(11)
    q = rng.integers(0, 20, 100, dtype=np.uint8)
    recs = random_records(rng, 20, 100, 1, 300, q)
    K = max(2, ((101 + G - 1) // G + 1) & ~1)
    if K > 64:
        pytest.skip("shape needs more than 64 columns per thread")
    ctx.set_option(native.OPT_WAVE_GROUP, G)
    ctx.set_option(native.OPT_WAVE_K, K)
    try:
        for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 15), (native.ALGO_SEMI_GLOBAL, 0),
                           (native.ALGO_LOCAL, 0)):
            g, o = run_both(ctx, algo, O.BLOSUM62, q, recs, 10, 1, ends)
            assert_same(g, o, f"G={G} K={K} algo={algo} ends={ends}")
    finally:
        ctx.set_option(native.OPT_WAVE_GROUP, 0)
        ctx.set_option(native.OPT_WAVE_K, 0)


@pytest.mark.parametrize("G,K", [(2, 52), (2, 64), (4, 50), (4, 64), (16, 64)])
def test_wide_rows(ctx, G, K):
    # wide rows (K > 48: 128 x 2 blocks for semi-global, 256 x 1 for local):
    # every end rule, records of unequal lengths in a pair (one lane ends rows
    # before the other) and empty ones
    rng = np.random.default_rng(19 + K)
    q = rng.integers(0, 20, 100, dtype=np.uint8)
    recs = random_records(rng, 20, 160, 0, 500, q)
    ctx.set_option(native.OPT_WAVE_GROUP, G)
    ctx.set_option(native.OPT_WAVE_K, K)
    try:
        for ends in ALL_ENDS:
            g, o = run_both(ctx, native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, recs, 10, 1, ends)
            assert_same(g, o, f"G={G} K={K} SG ends={ends}")
        g, o = run_both(ctx, native.ALGO_LOCAL, O.BLOSUM62, q, recs, 10, 1, 0)
        assert_same(g, o, f"G={G} K={K} SW")
    finally:
        ctx.set_option(native.OPT_WAVE_GROUP, 0)
        ctx.set_option(native.OPT_WAVE_K, 0)


@pytest.mark.parametrize("ext", [0, 1, 3, 200, 1000, 2048, 2049])
def test_semi_global_row_frames(ctx, ext):
    # semi-global rows are held in frames rising by ext per row and dropped
    # back every R rows (R * ext <= 2048): R = 2048 at ext 1, 8 at ext 200,
    # 2 at ext 1000, 1 at ext 2048 (a drop every row); ext 0 never moves the
    # frame; ext 2049 leaves the fast regime (exact kernels).  Records run
    # through many drops, every end rule, several group shapes.
    rng = np.random.default_rng(29 + ext)
    gap_open = ext + 7
    # query lengths that keep the fast regime's headroom check (about
    # 2 * open + ext * (padded Q + 3) <= 30000) so the frames are what runs
    shapes = {1000: ((12, 0), (20, 0)), 2048: ((5, 0), (8, 0))}.get(ext, ((40, 0), (40, 4), (120, 0)))
    for qlen, G in shapes:
        q = rng.integers(0, 20, qlen, dtype=np.uint8)
        recs = random_records(rng, 20, 60, 0, 700, q, plant_frac=0.4, sub=0.05)
        if G:
            ctx.set_option(native.OPT_WAVE_GROUP, G)
        try:
            for ends in ALL_ENDS:
                g, o = run_both(ctx, native.ALGO_SEMI_GLOBAL, O.BLOSUM62, q, recs, gap_open, ext, ends, thr=0.2)
                assert_same(g, o, f"ext={ext} Q={qlen} G={G} ends={ends}")
        finally:
            ctx.set_option(native.OPT_WAVE_GROUP, 0)


@pytest.mark.parametrize("K", [25, 28, 32, 34, 38, 44, 48])
def test_register_lean_builds(ctx, K):
    # both builds of a K (the register-lean one with fewer warps per SM, and
    # the default), single and batched launches, give the oracle's results
    rng = np.random.default_rng(23 + K)
    G = 4
    q = rng.integers(0, 20, G * K - 3, dtype=np.uint8)
    recs = random_records(rng, 20, 120, 0, 2 * len(q) + 30, q)
    ctx.set_option(native.OPT_WAVE_GROUP, G)
    ctx.set_option(native.OPT_WAVE_K, K)
    try:
        for lean in (0, 1):
            ctx.set_option(native.OPT_WAVE_LEAN, lean)
            for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 15), (native.ALGO_LOCAL, 0)):
                g, o = run_both(ctx, algo, O.BLOSUM62, q, recs, 10, 1, ends)
                assert_same(g, o, f"K={K} lean={lean} algo={algo} ends={ends}")
            m = ScoringMatrix(O.BLOSUM62)
            buf, off = native.pack_records(recs)
            sid = ctx.records_load(buf, off)
            qid = ctx.set_query(q, O.BLOSUM62, m.values, native.ALGO_LOCAL, 10, 1, 0, int(m.values[q, q].sum()), 0.5)
            try:
                single = ctx.score_set(qid, sid)
                batched = ctx.score_multi([qid], sid)
                for k in ("score", "qend", "tend"):
                    assert np.array_equal(single[k], batched[k][0]), f"K={K} lean={lean} batched {k}"
            finally:
                ctx.free_query(qid)
                ctx.records_free(sid)
    finally:
        ctx.set_option(native.OPT_WAVE_LEAN, -1)
        ctx.set_option(native.OPT_WAVE_GROUP, 0)
        ctx.set_option(native.OPT_WAVE_K, 0)


@pytest.mark.parametrize("kernel", [native.KERNEL_PLAIN, native.KERNEL_PLAIN16])
@pytest.mark.parametrize("algo", [native.ALGO_SEMI_GLOBAL, native.ALGO_LOCAL])
def test_plain_kernel_parity(ctx, algo, kernel):
    # both storage forms of the one-thread-per-record kernel: int32 columns in
    # global scratch, and int16 per-thread arrays (queries of 1 .. 2048
    # residues cover every array size, 2100 falls back to int32 columns)
    rng = np.random.default_rng(13)
    qlens = (150,) if kernel == native.KERNEL_PLAIN else (1, 64, 65, 150, 700, 2048, 2100)
    for qlen in qlens:
        q = rng.integers(0, 20, qlen, dtype=np.uint8)
        recs = random_records(rng, 20, 300 if qlen < 1000 else 60, 0, 400, q)
        for ends in ((12, 15, 0, 5) if algo == native.ALGO_SEMI_GLOBAL else (0,)):
            g, o = run_both(ctx, algo, O.BLOSUM62, q, recs, 10, 1, ends, kernel=kernel)
            assert_same(g, o, f"plain kernel={kernel} Q={qlen} algo={algo} ends={ends}")


def test_edge_cases(ctx):
    rng = np.random.default_rng(17)
    q = rng.integers(0, 5, 40, dtype=np.uint8)
    # empty records, length-1 records, odd count, one record only
    for recs in ([np.zeros(0, np.uint8)] * 3, [np.array([1], np.uint8)], random_records(rng, 5, 1, 1, 5),
                 random_records(rng, 5, 7, 0, 3) + [q.copy()]):
        for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 15), (native.ALGO_SEMI_GLOBAL, 0),
                           (native.ALGO_LOCAL, 0)):
            g, o = run_both(ctx, algo, O.ACTGN, q, recs, 3, 1, ends)
            assert_same(g, o, f"edge algo={algo} ends={ends} n={len(recs)}")


def test_empty_query(ctx):
    recs = [np.array([0, 1, 2], np.uint8), np.zeros(0, np.uint8)]
    g, o = run_both(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, np.zeros(0, np.uint8), recs, 3, 1, 12)
    assert (g["score"] == o["score"]).all() and (g["tend"] == o["tend"]).all()


def test_bad_record_code_is_an_error(ctx):
    m = ScoringMatrix(O.ACTGN)
    q = np.array([0, 1, 2, 3], np.uint8)
    qid = ctx.set_query(q, O.ACTGN, m.values, native.ALGO_SEMI_GLOBAL, 3, 1, 12, 8, 0.5)
    buf, off = native.pack_records([np.array([0, 9, 1], np.uint8)])
    with pytest.raises(native.IshGpuError) as e:
        ctx.score(qid, buf, off)
    assert e.value.code == native.EINVAL
    ctx.free_query(qid)
    # the context stays usable
    g, o = run_both(ctx, native.ALGO_SEMI_GLOBAL, O.ACTGN, q, [q.copy()], 3, 1, 12)
    assert_same(g, o, "after error")


def test_resident_set_matches_one_shot(ctx):
    rng = np.random.default_rng(19)
    q = rng.integers(0, 20, 300, dtype=np.uint8)
    recs = random_records(rng, 20, 500, 30, 900, q, plant_frac=0.05)
    buf, off = native.pack_records(recs)
    m = ScoringMatrix(O.BLOSUM62)
    mx = int(m.values[q, q].sum())
    sid = ctx.records_load(buf, off)
    assert ctx.records_info(sid) == (len(recs), len(buf))
    for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_LOCAL, 0)):
        qid = ctx.set_query(q, O.BLOSUM62, m.values, algo, 10, 1, ends, mx, 0.4)
        a = ctx.score(qid, buf, off)
        b = ctx.score_set(qid, sid)
        b2 = ctx.score_set(qid, sid)
        for k in ("score", "qend", "tend", "hit", "hit_idx"):
            assert (a[k] == b[k]).all() and (b[k] == b2[k]).all(), k
        ctx.free_query(qid)
    ctx.records_free(sid)


def test_matchers_on_reference_searcher_fixtures(ctx):
    """tests/test_searcher.mojo:77-200 through the GPU matchers."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from searcher_fixtures import cases, records, render

    for case in cases():
        for algo, ends in (("local", None), ("sg", "TTTT"), ("sg", "FFTT")):
            if algo == "sg":
                mt = StripedSemiGlobalMatcher(case["pattern"].encode(), 0.8, ends, case["matrix"], context=ctx)
            else:
                mt = StripedLocalMatcher(case["pattern"].encode(), 0.8, case["matrix"], context=ctx)
            recs = records(case)
            enc = [mt.convert_ascii_to_encoding(seq) for _, seq in recs]
            res = mt.batch_match(enc)
            got = render(case, recs, res.hit.astype(bool), mt.matrix.code_to_ascii, enc)
            exp = case["expected"]
            if case["record_type"] == "fastx":
                assert got.upper() == exp.upper(), (case["line"], algo, ends)
            else:
                assert got == exp, (case["line"], algo, ends)
            ctx.free_query(mt.query_id)


def test_reference_searcher_fixtures_from_text_split_on_the_device(ctx):
    """tests/test_searcher.mojo:77-200 end to end on the device: the fixture
    file's text split into line or FASTA records by the library
    (ish_gpu_records_load_lines / _fastx), scored, and the matched records
    written back from the device's copy (ish_gpu_records_get, names from the
    splitter's bounds) through the runners' output writer."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from searcher_fixtures import cases

    from ish_gb300 import output

    for case in cases():
        text = case["in_data"].encode()
        for algo, ends in (("local", None), ("sg", "TTTT"), ("sg", "FFTT")):
            if algo == "sg":
                mt = StripedSemiGlobalMatcher(case["pattern"].encode(), 0.8, ends, case["matrix"], context=ctx)
            else:
                mt = StripedLocalMatcher(case["pattern"].encode(), 0.8, case["matrix"], context=ctx)
            if case["record_type"] == "line":
                sid, n = ctx.records_load_lines(text, mt.matrix.kind)
                bounds = None
            else:
                sid, n, bounds = ctx.records_load_fastx(text, mt.matrix.kind)
            try:
                hits = ctx.score_set(mt.query_id, sid)["hit_idx"]
                codes, off = ctx.records_get(sid)
            finally:
                ctx.records_free(sid)
            matches = [(int(i), 0, 0) for i in hits]
            parts = []
            if case["record_type"] == "line":
                output.write_line_matches(parts.append, codes, off, matches, mt.matrix.code_to_ascii)
            else:
                names = [text[int(b[0]):int(b[1])] for b in bounds]
                output.write_fastx_matches(parts.append, names, codes, off, matches, mt.matrix.code_to_ascii)
            got = b"".join(parts).decode("utf-8", errors="surrogateescape")
            exp = case["expected"]
            if case["record_type"] == "fastx":
                assert got.upper() == exp.upper(), (case["line"], algo, ends)
            else:
                assert got == exp, (case["line"], algo, ends)
            ctx.free_query(mt.query_id)


@pytest.mark.parametrize("layout", [native.PROF_S16, native.PROF_PAIR, native.PROF_S32])
@pytest.mark.parametrize("kind", [O.ACTGN, O.BLOSUM62])
def test_every_profile_layout(ctx, layout, kind):
    # the three shared-memory profile layouts give identical results
    rng = np.random.default_rng(3000 + 10 * layout + kind)
    alpha = 5 if kind == O.ACTGN else 20
    # (the pair layout of a 24-letter alphabet holds 576 rows: short queries
    # keep it within shared memory)
    for qlen in ((13, 40, 97) if kind == O.ACTGN else (13, 40)):
        q = rng.integers(0, alpha, qlen, dtype=np.uint8)
        recs = random_records(rng, alpha, 150, 0, 2 * qlen + 30, q)
        ctx.set_option(native.OPT_PROFILE_LAYOUT, layout)
        try:
            for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 5), (native.ALGO_LOCAL, 0)):
                g, o = run_both(ctx, algo, kind, q, recs, 10 if kind == O.BLOSUM62 else 3, 1, ends)
                assert_same(g, o, f"layout={layout} kind={kind} Q={qlen} algo={algo} ends={ends}")
        finally:
            ctx.set_option(native.OPT_PROFILE_LAYOUT, native.PROF_AUTO)


@pytest.mark.parametrize("qlen", [120, 300, 1000])
def test_ascii_long_queries(ctx, qlen):
    # 256-code ascii profiles: codes absent from the query share one profile
    # row, which keeps long ascii queries within shared memory
    rng = np.random.default_rng(4000 + qlen)
    printable = np.arange(0x20, 0x7F, dtype=np.uint8)
    q = rng.choice(printable, qlen)
    recs = [rng.choice(printable, int(rng.integers(0, 2 * qlen))) for _ in range(120)]
    for r in recs[::5]:
        if len(r) >= qlen:
            pos = int(rng.integers(0, len(r) - qlen + 1))
            r[pos:pos + qlen] = q
    for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 3), (native.ALGO_LOCAL, 0)):
        g, o = run_both(ctx, algo, O.ASCII, q, recs, 3, 1, ends, thr=0.6)
        assert_same(g, o, f"ascii Q={qlen} algo={algo} ends={ends}")


def test_calibration_kernels_report_rates(ctx):
    # the integer-roofline calibration and the lane-width microbenchmark run
    # and report finite, positive rates
    assert 1e11 < ctx.calibrate() < 1e15
    lanes = ctx.calibrate_lanes()
    for k in ("s16x2_cells_per_s", "u8x4_cells_per_s"):
        assert 1e10 < lanes[k] < 1e16, lanes

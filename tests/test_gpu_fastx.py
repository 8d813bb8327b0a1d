"""FASTA/FASTQ records split on the device (ish_gpu_records_load_fastx) against
the oracle's byte-level restatement of ish's reader (oracle/fastx.py,
ishlib/vendor/kseq.mojo:370-461): the same records, names, qualities and
sequences, and a refusal exactly where the reader would continue a quality on
the next line.  Sequences come back through ish_gpu_records_get."""
import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import ScoringMatrix
from oracle.fastx import read_records
from test_fastx_cpu import random_text

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    native.load(build_if_missing=True)
    c = native.Context(0)
    yield c
    c.close()


def device_records(ctx, data, kind=O.ASCII):
    sid, n, bounds = ctx.records_load_fastx(data, kind)
    try:
        assert ctx.records_info(sid)[0] == n
        codes, off = ctx.records_get(sid)
    finally:
        ctx.records_free(sid)
    out = []
    for i in range(n):
        ns, ne, qs, qe = (int(x) for x in bounds[i])
        seq = codes[int(off[i]):int(off[i + 1])].tobytes()
        out.append((data[ns:ne], seq, data[qs:qe] if qe > qs else None))
    return out


def check(ctx, data):
    want, continued = read_records(data, with_continued=True)
    if continued:
        with pytest.raises(native.IshGpuError) as e:
            ctx.records_load_fastx(data, O.ASCII)
        assert e.value.code == native.EINVAL
        return
    got = device_records(ctx, data)
    # a FASTQ record with an empty quality has no quality bounds: compare as empty
    want = [(nm, sq, q if q else None) for nm, sq, q in want]
    assert got == want, data


HANDWRITTEN = [
    b">a x\nACGT\nAC\r\n>b\nGG\n",
    b"@r1\nACGT\n+\n@III\n@r2\nAC\n+r2\nII\n",
    b"junk>h1\nAC\n>h2\nTT",
    b">a\nAC\n\n>b\nGG\n",
    b">a\nAC\n>b\n>c\nT\n",
    b"@r1\nAC\n+\nIII\n@r2\nA\n+\nI\n",
    b"@r1\nACGT\n+\nII\nII\n",
    b"@r1\nAC\n+\n",
    b">a\nAC\n>",
    b"\r\r>a\r\n\rAC\r\n\r\n",
    b">a\nAC\n@q\nGT\n+\nII\n>c\nA\n",
    b"\n\n\n", b"no header at all\n", b">", b"@",
]


def test_handwritten_files(ctx):
    for data in HANDWRITTEN:
        check(ctx, data)


def test_empty_text(ctx):
    sid, n, b = ctx.records_load_fastx(b"", O.ASCII)
    assert n == 0 and len(b) == 0
    ctx.records_free(sid)


def test_random_texts(ctx):
    rng = np.random.default_rng(77)
    for _ in range(400):
        check(ctx, random_text(rng, int(rng.integers(1, 60))))


def _fasta(rng, n, width):
    recs, parts = [], []
    for i in range(n):
        s = rng.choice(np.frombuffer(b"ACGTN", np.uint8), int(rng.integers(1, 700))).tobytes()
        recs.append((f"rec{i} some comment".encode(), s))
        parts.append(b">" + recs[-1][0] + b"\n" + b"\n".join(s[k:k + width] for k in range(0, len(s), width)) + b"\n")
    return b"".join(parts), recs


def _fastq(rng, n):
    parts, recs = [], []
    for i in range(n):
        s = rng.choice(np.frombuffer(b"ACGT", np.uint8), int(rng.integers(100, 301))).tobytes()
        q = rng.integers(33, 75, len(s), dtype=np.uint8).tobytes()  # includes '@' (64) and '>' (62)
        recs.append((f"read{i}".encode(), s, q))
        parts.append(b"@" + recs[-1][0] + b"\n" + s + b"\n+\n" + q + b"\n")
    return b"".join(parts), recs


def test_large_fasta_and_fastq_match_the_reader(ctx):
    rng = np.random.default_rng(5)
    for data in (_fasta(rng, 3000, 60)[0], _fastq(rng, 20000)[0]):
        want = read_records(data)
        got = device_records(ctx, data)
        assert len(got) == len(want)
        assert got == [(nm, sq, q if q else None) for nm, sq, q in want]


def test_scores_equal_records_loaded_from_host(ctx):
    # FASTQ reads encoded on the device (actgn) score exactly as the same
    # reads encoded by the host's table and loaded as records
    rng = np.random.default_rng(9)
    data, recs = _fastq(rng, 5000)
    m = ScoringMatrix(O.ACTGN)
    sid, n, _ = ctx.records_load_fastx(data, O.ACTGN)
    assert n == len(recs)
    buf, off = native.pack_records([m.encode(s) for _, s, _ in recs])
    sid2 = ctx.records_load(buf, off)
    q = m.encode(b"ACGTTGCAACGTAGCTAGCTAGGCTAGCATCGATCGA")
    qid = ctx.set_query(q, O.ACTGN, m.values, native.ALGO_SEMI_GLOBAL, 3, 1,
                        native.FREE_TARGET_START | native.FREE_TARGET_END, int(m.values[q, q].sum()), 0.5)
    a = ctx.score_set(qid, sid)
    b = ctx.score_set(qid, sid2)
    for k in ("score", "qend", "tend", "hit"):
        assert np.array_equal(a[k], b[k]), k
    o = O.Matcher(O.SEMI_GLOBAL, O.ACTGN, q, int(m.values[q, q].sum()), 0.5, gap_open=3, gap_extend=1,
                  ends=O.TS | O.TE).batch(buf, off, threads=4)
    assert np.array_equal(a["score"], o["score"]) and np.array_equal(a["hit"], o["hit"])
    ctx.free_query(qid)
    ctx.records_free(sid)
    ctx.records_free(sid2)


def test_bounds_capacity_is_checked(ctx):
    data = b">a\nAC\n>b\nGG\n"
    buf = np.frombuffer(data, np.uint8)
    import ctypes as C

    sid, n = C.c_int32(), C.c_uint32()
    bnd = np.zeros((1, 4), np.uint64)
    rc = ctx._L.ish_gpu_records_load_fastx(ctx._h, buf.ctypes.data_as(C.POINTER(C.c_uint8)), len(buf), O.ASCII,
                                            C.byref(sid), C.byref(n), bnd.ctypes.data_as(C.POINTER(C.c_uint64)), 1)
    assert rc == native.EOVERFLOW
    # the context stays usable
    check(ctx, data)


def test_records_get_ranges(ctx):
    rng = np.random.default_rng(3)
    recs = [rng.integers(0, 20, int(rng.integers(0, 50)), dtype=np.uint8) for _ in range(300)]
    buf, off = native.pack_records(recs)
    sid = ctx.records_load(buf, off)
    for first, count in ((0, 300), (17, 40), (299, 1), (5, 0)):
        codes, o = ctx.records_get(sid, first, count)
        for i in range(count):
            assert np.array_equal(codes[int(o[i]):int(o[i + 1])], recs[first + i])
    with pytest.raises(native.IshGpuError):
        ctx.records_get(sid, 250, 60)
    ctx.records_free(sid)


def test_packing_round_trip_short_and_long_records(ctx):
    """Every record, as packed on the device, read back byte for byte: short
    records (copied by lane groups sized to the set's average length), records
    of 16 KB and more (copied by whole blocks, longest first) and empty ones,
    at odd offsets in the caller's buffer (the pack realigns every record),
    with and without the device-side encoding of raw text."""
    rng = np.random.default_rng(41)
    lens = ([int(x) for x in rng.integers(0, 200, 3000)] + [0, 1, 15, 16, 17, 16383, 16384, 16385]
            + [int(x) for x in rng.integers(16384, 300_000, 12)])
    rng.shuffle(lens)
    recs = [rng.integers(0, 20, L, dtype=np.uint8) for L in lens]
    buf, off = native.pack_records(recs)
    # a caller's buffer whose records start 3 bytes into it
    shifted = np.concatenate([np.full(3, 99, np.uint8), buf])
    for b, o in ((buf, off), (shifted, off + np.uint64(3))):
        sid = ctx.records_load(b, o)
        codes, got = ctx.records_get(sid)
        ctx.records_free(sid)
        for i, r in enumerate(recs):
            assert np.array_equal(codes[int(got[i]):int(got[i + 1])], r), (i, len(r))
    # raw residues encoded on the device (blosum62 letters -> codes)
    letters = ScoringMatrix(O.BLOSUM62).code_to_ascii
    raw = [letters[r] for r in recs]
    rbuf, roff = native.pack_records(raw)
    sid = ctx.records_load_raw(rbuf, roff, O.BLOSUM62)
    codes, got = ctx.records_get(sid)
    ctx.records_free(sid)
    for i, r in enumerate(recs):
        assert np.array_equal(codes[int(got[i]):int(got[i + 1])], r), ("raw", i, len(r))

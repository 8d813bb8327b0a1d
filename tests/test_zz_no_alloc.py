"""ish_gpu_score_noalloc against ish_gpu_score (collected last on purpose).

ish_gpu_score_noalloc is for callers that cannot allocate device memory when
they score: their device memory belongs to another allocator or a fixed arena,
or their host forbids cudaMalloc/cudaFree from the scoring thread.  It scores
records the caller already holds in device memory into device outputs the
caller owns, using only the library's fixed 32 MiB __device__ scratch array.

This test places records and outputs in device memory (allocated here, by the
test, through torch), calls the entry point through the C ABI twice in a row
(the second call runs on the scratch contents the first one left behind) and
requires the results to equal ish_gpu_score's exactly -- scores are integers,
so the tolerance is zero -- for semi-global and local scoring.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import BLOSUM62, ScoringMatrix

pytestmark = pytest.mark.gpu


def _records(seed, q):
    rng = np.random.default_rng(seed)
    recs = []
    for i in range(300):
        r = rng.integers(0, 20, int(rng.integers(0, 500)), dtype=np.uint8)
        if i % 7 == 0 and len(r) >= len(q):
            pos = int(rng.integers(0, len(r) - len(q) + 1))
            r[pos:pos + len(q)] = q
        recs.append(r)
    return native.pack_records(recs)


def _noalloc(lib, torch, d_recs, nbytes, d_off, n, q, m, algo, ends, mx, thr, outs, stream, gap_open=10,
             gap_ext=1):
    err = C.create_string_buffer(256)
    qa = np.ascontiguousarray(q, np.uint8)
    mv = np.ascontiguousarray(m.values.ravel(), np.int8)
    rc = lib.ish_gpu_score_noalloc(
        C.c_void_p(d_recs.data_ptr()), nbytes, C.c_void_p(d_off.data_ptr()), n,
        qa.ctypes.data_as(C.POINTER(C.c_uint8)) if len(qa) else None, len(qa),
        mv.ctypes.data_as(C.POINTER(C.c_int8)), m.size, algo, gap_open, gap_ext, ends, mx, thr,
        *(C.c_void_p(o.data_ptr()) for o in outs), C.c_void_p(stream), err, len(err))
    return rc, err.value.decode()


def _device(torch, buf, off):
    n = len(off) - 1
    d_recs = torch.from_numpy(buf.copy() if len(buf) else np.zeros(16, np.uint8)).cuda()
    d_off = torch.from_numpy(off.view(np.int64).copy()).cuda()
    outs = [torch.empty(max(n, 1), dtype=torch.int32, device="cuda") for _ in range(3)] + \
           [torch.empty(max(n, 1), dtype=torch.uint8, device="cuda")]
    return d_recs, d_off, outs


def _oracle(buf, off, q, algo, ends, mx, thr):
    om = O.Matcher(O.SEMI_GLOBAL if algo == native.ALGO_SEMI_GLOBAL else O.LOCAL, BLOSUM62, q, mx, thr,
                   gap_open=10, gap_extend=1, ends=ends)
    return om.batch(buf, off, threads=os.cpu_count() or 4)


def test_noalloc_matches_score_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = native.load(build_if_missing=True)
    m = ScoringMatrix(BLOSUM62)
    rng = np.random.default_rng(42)
    q = rng.integers(0, 20, 150, dtype=np.uint8)
    mx = int(m.values[q, q].sum())
    buf, off = _records(7, q)
    n = len(off) - 1
    d_recs = torch.from_numpy(buf.copy()).cuda()
    d_off = torch.from_numpy(off.view(np.int64).copy()).cuda()
    outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(3)] + \
           [torch.empty(n, dtype=torch.uint8, device="cuda")]
    stream = torch.cuda.current_stream().cuda_stream
    with native.Context(0) as ctx:
        for algo, ends in ((native.ALGO_SEMI_GLOBAL, native.FREE_TARGET_START | native.FREE_TARGET_END),
                           (native.ALGO_SEMI_GLOBAL, 15), (native.ALGO_LOCAL, 0)):
            qid = ctx.set_query(q, BLOSUM62, m.values, algo, 10, 1, ends, mx, 0.5)
            ref = ctx.score(qid, buf, off)
            ctx.free_query(qid)
            for call in range(2):
                for o in outs:
                    o.fill_(7)
                rc, msg = _noalloc(lib, torch, d_recs, len(buf), d_off, n, q, m, algo, ends, mx, 0.5, outs, stream)
                assert rc == 0, msg
                got = [o.cpu().numpy() for o in outs]
                for name, g, r in zip(("score", "qend", "tend", "hit"), got,
                                      (ref["score"], ref["qend"], ref["tend"], ref["hit"])):
                    assert (g == r).all(), f"{name} differs (algo {algo}, ends {ends}, call {call})"
            # and directly against the oracle (the CPU restatement of ish's matchers)
            o = _oracle(buf, off, q, algo, ends, mx, 0.5)
            for name, g in zip(("score", "qend", "tend", "hit"), got):
                assert (g == o[name]).all(), f"{name} differs from the oracle (algo {algo}, ends {ends})"


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = native.load(build_if_missing=True)
    m = ScoringMatrix(0)  # ascii: 256 x 256
    q = np.full(30000, 65, np.uint8)
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    d_off = torch.zeros(2, dtype=torch.int64, device="cuda")
    outs = [torch.empty(1, dtype=torch.int32, device="cuda") for _ in range(3)] + \
           [torch.empty(1, dtype=torch.uint8, device="cuda")]
    rc, msg = _noalloc(lib, torch, d, 16, d_off, 1, q, m, native.ALGO_SEMI_GLOBAL, 12, 2 * len(q), 0.5, outs, 0)
    assert rc == native.EOVERFLOW
    assert "scratch" in msg


def test_noalloc_edge_cases_against_the_oracle():
    """An empty query and empty records are scored as the oracle scores them;
    what the entry point cannot score exactly is refused, not approximated:
    gap_open <= gap_extend, a record too long for the int16 boundary row when
    the target start is fixed, and offsets that run backwards."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    lib = native.load(build_if_missing=True)
    m = ScoringMatrix(BLOSUM62)
    rng = np.random.default_rng(5)
    recs = [rng.integers(0, 20, int(rng.integers(0, 60)), dtype=np.uint8) for _ in range(40)] + [np.zeros(0, np.uint8)]
    buf, off = native.pack_records(recs)
    n = len(off) - 1
    d_recs, d_off, outs = _device(torch, buf, off)
    for q in (np.zeros(0, np.uint8), rng.integers(0, 20, 1, dtype=np.uint8), rng.integers(0, 20, 33, dtype=np.uint8)):
        mx = int(m.values[q, q].sum()) if len(q) else 0
        for algo, ends in ((native.ALGO_SEMI_GLOBAL, 12), (native.ALGO_SEMI_GLOBAL, 0), (native.ALGO_SEMI_GLOBAL, 15),
                           (native.ALGO_LOCAL, 0)):
            rc, msg = _noalloc(lib, torch, d_recs, len(buf), d_off, n, q, m, algo, ends, mx, 0.3, outs, 0)
            assert rc == 0, msg
            o = _oracle(buf, off, q, algo, ends, mx, 0.3)
            for name, d in zip(("score", "qend", "tend", "hit"), outs):
                g = d.cpu().numpy()[:n]
                assert (g == o[name]).all(), f"{name}: Q={len(q)} algo={algo} ends={ends}"
    q = rng.integers(0, 20, 150, dtype=np.uint8)
    mx = int(m.values[q, q].sum())
    # gap_open <= gap_extend: outside the exact-integer regime
    rc, msg = _noalloc(lib, torch, d_recs, len(buf), d_off, n, q, m, native.ALGO_SEMI_GLOBAL, 12, mx, 0.5, outs, 0,
                       gap_open=1, gap_ext=1)
    assert rc == native.EINVAL and "regime" in msg
    # a fixed target start on a 30,000-residue record: its boundary row leaves int16
    long_buf, long_off = native.pack_records([rng.integers(0, 20, 30000, dtype=np.uint8)])
    d_l, d_lo, outs_l = _device(torch, long_buf, long_off)
    rc, msg = _noalloc(lib, torch, d_l, len(long_buf), d_lo, 1, q, m, native.ALGO_SEMI_GLOBAL, 0, mx, 0.5, outs_l, 0)
    assert rc == native.EINVAL and "too long" in msg
    # ... which a free target start scores exactly
    rc, msg = _noalloc(lib, torch, d_l, len(long_buf), d_lo, 1, q, m, native.ALGO_SEMI_GLOBAL, 12, mx, 0.5, outs_l, 0)
    assert rc == 0, msg
    o = _oracle(long_buf, long_off, q, native.ALGO_SEMI_GLOBAL, 12, mx, 0.5)
    assert int(outs_l[0].cpu()[0]) == int(o["score"][0]) and int(outs_l[2].cpu()[0]) == int(o["tend"][0])
    # offsets that run backwards
    bad = torch.tensor([0, 40, 20, 60], dtype=torch.int64, device="cuda")
    rc, msg = _noalloc(lib, torch, d_recs, len(buf), bad, 3, q, m, native.ALGO_LOCAL, 0, mx, 0.5, outs, 0)
    assert rc == native.EINVAL and "offsets" in msg

"""CPU oracle for ish's striped alignment-scoring path.

TEST INFRASTRUCTURE ONLY.  This package is the parity checker for the CUDA path
and the timed CPU baseline of ``bench.py``.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import it; the
product (``ish_gb300`` and ``libish_gpu.so``) never does.

The C sources (``ish_oracle.c``) restate the reference's Mojo implementation
line by line; see the citations there.  This module is a thin ctypes layer.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libish_oracle.so")

ASCII, ACTGN, ACTGN0, BLOSUM62 = 0, 1, 2, 3
SEMI_GLOBAL, LOCAL = 0, 1
QS, QE, TS, TE = 1, 2, 4, 8

MATRIX_NAMES = {"ascii": ASCII, "actgn": ACTGN, "actgn0": ACTGN0, "blosum62": BLOSUM62}


def ends_from_str(s: str) -> int:
    """(query_start, query_end, target_start, target_end) as 'FFTT'."""
    s = s.upper()
    assert len(s) == 4 and set(s) <= {"T", "F"}
    return sum(bit for bit, ch in zip((QS, QE, TS, TE), s) if ch == "T")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("ish_oracle.c", "ish_oracle_neon.c", "ish_oracle.h")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, srcs)):
        # -B: rebuild even when make's timestamps say otherwise (force, or a
        # copy of the tree with reset times)
        r = subprocess.run(["make", "-s", "-B", "-C", HERE, "libish_oracle.so"], capture_output=True, text=True)
        if r.returncode != 0:
            # the NEON passes did not compile: the lane loops alone
            sys.stderr.write("oracle: vector passes not built (%s); lane loops only\n" % r.stderr.strip()[-400:])
            subprocess.check_call(["make", "-s", "-B", "-C", HERE, "libish_oracle.so", "EXTRA=-DISH_O_NO_NEON"])
    return LIB_PATH


def set_vectors(on: bool) -> None:
    """On an aarch64 host, run the striped passes on NEON vectors (default)
    or on the lane loops (for comparing the two)."""
    lib().ish_o_set_vectors(1 if on else 0)


def vectors() -> bool:
    """Whether the striped passes run on NEON vectors."""
    return bool(lib().ish_o_vectors())


class End(C.Structure):
    _fields_ = [("score", C.c_int32), ("reference", C.c_int32), ("query", C.c_int32)]

    def tuple(self):
        return (self.score, self.reference, self.query)


class StartEnd(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score", "query_start", "query_end", "target_start", "target_end")]


class Alignment(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score1", "ref_begin1", "ref_end1", "read_begin1", "read_end1", "used_word")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        u8p, i8p, i16p, u16p = (C.POINTER(t) for t in (C.c_uint8, C.c_int8, C.c_int16, C.c_uint16))
        L.ish_o_matrix.argtypes = [C.c_int, C.POINTER(i8p), C.POINTER(u8p), C.POINTER(u8p)]
        L.ish_o_matrix.restype = C.c_int
        L.ish_o_encode_and_score.argtypes = [C.c_int, u8p, C.c_size_t, u8p]
        L.ish_o_encode_and_score.restype = C.c_int32
        L.ish_o_sg_profile_i16.argtypes = [u8p, C.c_int, i8p, C.c_int, C.c_int, i16p]
        L.ish_o_sg_profile_i8.argtypes = [u8p, C.c_int, i8p, C.c_int, C.c_int, i8p]
        L.ish_o_sw_profile_u8.argtypes = [u8p, C.c_int, i8p, C.c_int, C.c_int, C.c_uint8, u8p]
        L.ish_o_sw_profile_u16.argtypes = [u8p, C.c_int, i8p, C.c_int, C.c_int, C.c_uint8, u16p]
        L.ish_o_matrix_minmax.argtypes = [i8p, C.c_int, i8p, i8p]
        L.ish_o_sw_bias.argtypes = [i8p, C.c_int]
        L.ish_o_sw_bias.restype = C.c_uint8
        L.ish_o_set_vectors.argtypes = [C.c_int]
        L.ish_o_vectors.restype = C.c_int
        L.ish_o_sg_aln_i16.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_int, i16p, C.c_int, C.c_int8, C.c_int8, C.c_int]
        L.ish_o_sg_aln_i16.restype = End
        L.ish_o_sg_aln_i8.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_int, i8p, C.c_int, C.c_int8, C.c_int8, C.c_int]
        L.ish_o_sg_aln_i8.restype = End
        L.ish_o_sg_start_end_i16.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_int, i16p, i16p, C.c_int,
                                             C.c_int8, C.c_int8, C.c_int, C.c_float, C.POINTER(StartEnd)]
        L.ish_o_sg_start_end_i16.restype = C.c_int
        L.ish_o_sw_u8.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint8, C.c_uint8, u8p, C.c_int, C.c_uint8, C.c_uint8]
        L.ish_o_sw_u8.restype = End
        L.ish_o_sw_u16.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint16, C.c_uint16, u16p, C.c_int, C.c_uint16, C.c_uint16]
        L.ish_o_sw_u16.restype = End
        L.ish_o_ssw_align.argtypes = [u8p, C.c_int, C.c_int, u8p, u16p, u8p, u16p, C.c_int, C.c_int, C.c_uint8,
                                      C.c_uint8, C.c_uint8, C.c_float, C.POINTER(Alignment)]
        L.ish_o_ssw_align.restype = C.c_int
        L.ish_o_matcher_new.argtypes = [C.c_int, C.c_int, u8p, C.c_int, C.c_int32, C.c_float, C.c_int, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_int]
        L.ish_o_matcher_new.restype = C.c_void_p
        L.ish_o_matcher_free.argtypes = [C.c_void_p]
        L.ish_o_matcher_forward.argtypes = [C.c_void_p, u8p, C.c_int]
        L.ish_o_matcher_forward.restype = End
        L.ish_o_matcher_first_match.argtypes = [C.c_void_p, u8p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.ish_o_matcher_first_match.restype = C.c_int
        L.ish_o_sg_find_start.argtypes = [C.c_void_p, u8p, C.c_int]
        L.ish_o_sg_find_start.restype = C.c_int64
        i32p, i64p, u64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_uint64)
        L.ish_o_matcher_batch.argtypes = [C.c_void_p, u8p, u64p, C.c_int64, C.c_int, i32p, i32p, i32p, u8p, i64p, i64p]
        L.ish_o_sg_model.argtypes = [u8p, C.c_int, u8p, C.c_int, i8p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ish_o_sg_model.restype = End
        L.ish_o_sw_model.argtypes = [u8p, C.c_int, u8p, C.c_int, i8p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ish_o_sw_model.restype = End
        _lib = L
    return _lib


def _u8(a):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint8))


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def matrix(kind: int):
    """(values int8[size*size], size, ascii_to_code uint8[256], code_to_ascii uint8[size])."""
    L = lib()
    v, a2c, c2a = C.POINTER(C.c_int8)(), C.POINTER(C.c_uint8)(), C.POINTER(C.c_uint8)()
    size = L.ish_o_matrix(kind, C.byref(v), C.byref(a2c), C.byref(c2a))
    vals = np.ctypeslib.as_array(v, shape=(size * size,)).copy()
    return vals, size, np.ctypeslib.as_array(a2c, shape=(256,)).copy(), np.ctypeslib.as_array(c2a, shape=(size,)).copy()


def encode_and_score(kind: int, text: bytes):
    buf, p = _u8(np.frombuffer(text, dtype=np.uint8) if len(text) else np.zeros(0, np.uint8))
    out = np.zeros(max(len(text), 1), np.uint8)
    score = lib().ish_o_encode_and_score(kind, p, len(text), _ptr(out, C.c_uint8))
    return out[: len(text)].copy(), int(score)


def encode(kind: int, text: bytes) -> np.ndarray:
    return encode_and_score(kind, text)[0]


def matrix_minmax(kind: int):
    vals, size, _, _ = matrix(kind)
    return int(min(0, vals.min())), int(max(0, vals.max()))


def sg_profile(q, kind: int, W: int, dtype=np.int16):
    vals, size, _, _ = matrix(kind)
    q, qp = _u8(q)
    seg = (len(q) + W - 1) // W
    out = np.zeros(max(size * seg * W, 1), dtype)
    fn = lib().ish_o_sg_profile_i16 if dtype == np.int16 else lib().ish_o_sg_profile_i8
    ct = C.c_int16 if dtype == np.int16 else C.c_int8
    fn(qp, len(q), _ptr(vals, C.c_int8), size, W, _ptr(out, ct))
    return out


def sg_aln(rec, q, kind, open_, ext, ends, W=8, dtype=np.int16):
    """semi_global_aln with a profile built from q."""
    prof = sg_profile(q, kind, W, dtype)
    mn, mx = matrix_minmax(kind)
    rec, rp = _u8(rec)
    if dtype == np.int16:
        r = lib().ish_o_sg_aln_i16(rp, len(rec), len(q), open_, ext, _ptr(prof, C.c_int16), W, mx, mn, ends)
    else:
        r = lib().ish_o_sg_aln_i8(rp, len(rec), len(q), open_, ext, _ptr(prof, C.c_int8), W, mx, mn, ends)
    return r.tuple()


def sg_start_end(rec, q, kind, open_, ext, ends, W=8, cutoff=float("-inf")):
    prof = sg_profile(q, kind, W)
    rprof = sg_profile(np.ascontiguousarray(np.asarray(q, np.uint8)[::-1]), kind, W)
    mn, mx = matrix_minmax(kind)
    rec, rp = _u8(rec)
    out = StartEnd()
    ok = lib().ish_o_sg_start_end_i16(rp, len(rec), len(q), open_, ext, _ptr(prof, C.c_int16),
                                      _ptr(rprof, C.c_int16), W, mx, mn, ends, cutoff, C.byref(out))
    if not ok:
        return None
    return dict(score=out.score, query_start=out.query_start, query_end=out.query_end,
                target_start=out.target_start, target_end=out.target_end)


def sw_profiles(q, kind, w_u8=16, w_u16=8):
    vals, size, _, _ = matrix(kind)
    bias = int(lib().ish_o_sw_bias(_ptr(vals, C.c_int8), size))
    q, qp = _u8(q)
    s8, s16 = (len(q) + w_u8 - 1) // w_u8, (len(q) + w_u16 - 1) // w_u16
    p8 = np.zeros(max(size * s8 * w_u8, 1), np.uint8)
    p16 = np.zeros(max(size * s16 * w_u16, 1), np.uint16)
    lib().ish_o_sw_profile_u8(qp, len(q), _ptr(vals, C.c_int8), size, w_u8, bias, _ptr(p8, C.c_uint8))
    lib().ish_o_sw_profile_u16(qp, len(q), _ptr(vals, C.c_int8), size, w_u16, bias, _ptr(p16, C.c_uint16))
    return p8, p16, bias


def sw(rec, q, kind, open_, ext, word=False, reverse=False, terminate=-1, W=None):
    p8, p16, bias = sw_profiles(q, kind, W or 16, W or 8)
    rec, rp = _u8(rec)
    if word:
        r = lib().ish_o_sw_u16(rp, len(rec), int(reverse), len(q), open_, ext, _ptr(p16, C.c_uint16),
                               W or 8, terminate & 0xFFFF, bias)
    else:
        r = lib().ish_o_sw_u8(rp, len(rec), int(reverse), len(q), open_, ext, _ptr(p8, C.c_uint8),
                              W or 16, terminate & 0xFF, bias)
    return r.tuple()


def ssw_align(rec, q, kind, open_, ext, cutoff=0.0, w_u8=16, w_u16=8):
    p8, p16, bias = sw_profiles(q, kind, w_u8, w_u16)
    rq = np.ascontiguousarray(np.asarray(q, np.uint8)[::-1])
    rp8, rp16, _ = sw_profiles(rq, kind, w_u8, w_u16)
    rec, rp = _u8(rec)
    out = Alignment()
    ok = lib().ish_o_ssw_align(rp, len(rec), len(q), _ptr(p8, C.c_uint8), _ptr(p16, C.c_uint16),
                               _ptr(rp8, C.c_uint8), _ptr(rp16, C.c_uint16), w_u8, w_u16, bias,
                               open_, ext, cutoff, C.byref(out))
    if not ok:
        return None
    return dict(score1=out.score1, ref_begin1=out.ref_begin1, ref_end1=out.ref_end1,
                read_begin1=out.read_begin1, read_end1=out.read_end1, used_word=out.used_word)


def sg_model(rec, q, kind, open_, ext, ends, W=8):
    vals, size, _, _ = matrix(kind)
    rec, rp = _u8(rec)
    q, qp = _u8(q)
    return lib().ish_o_sg_model(rp, len(rec), qp, len(q), _ptr(vals, C.c_int8), size, open_, ext, W, ends).tuple()


def sw_model(rec, q, kind, open_, ext, W=16):
    vals, size, _, _ = matrix(kind)
    rec, rp = _u8(rec)
    q, qp = _u8(q)
    return lib().ish_o_sw_model(rp, len(rec), qp, len(q), _ptr(vals, C.c_int8), size, open_, ext, W).tuple()


class Matcher:
    """StripedSemiGlobalMatcher / StripedLocalMatcher over an encoded pattern."""

    def __init__(self, algo, kind, enc_pattern, max_score, threshold, gap_open=3, gap_extend=1,
                 ends=TS | TE, w_sg=8, w_u8=16, w_u16=8):
        self.enc, p = _u8(enc_pattern if len(enc_pattern) else np.zeros(0, np.uint8))
        self._h = lib().ish_o_matcher_new(algo, kind, p, len(self.enc), int(max_score), float(threshold),
                                          int(gap_open), int(gap_extend), int(ends), w_sg, w_u8, w_u16)

    @classmethod
    def from_ascii(cls, algo, kind, pattern: bytes, threshold, **kw):
        enc, score = encode_and_score(kind, pattern)
        return cls(algo, kind, enc, score, threshold, **kw)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ish_o_matcher_free(self._h)
            self._h = None

    def forward(self, rec):
        rec, rp = _u8(rec)
        return lib().ish_o_matcher_forward(self._h, rp, len(rec)).tuple()

    def first_match(self, rec):
        rec, rp = _u8(rec)
        s, e = C.c_int64(), C.c_int64()
        if lib().ish_o_matcher_first_match(self._h, rp, len(rec), C.byref(s), C.byref(e)):
            return (s.value, e.value)
        return None

    def find_start(self, rec, end_exclusive):
        rec, rp = _u8(rec)
        return int(lib().ish_o_sg_find_start(self._h, rp, int(end_exclusive)))

    def batch(self, recs: np.ndarray, offsets: np.ndarray, threads: int = 1, forward=True, matches=True):
        """Per-record forward (score, qend, tend) and first_match (hit, start, end)."""
        n = len(offsets) - 1
        recs = np.ascontiguousarray(recs, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        out = {}
        i32 = lambda: np.zeros(max(n, 1), np.int32)
        if forward:
            out.update(score=i32(), qend=i32(), tend=i32())
        if matches:
            out.update(hit=np.zeros(max(n, 1), np.uint8), start=np.zeros(max(n, 1), np.int64),
                       end=np.zeros(max(n, 1), np.int64))
        g = lambda k, ct: _ptr(out[k], ct) if k in out else None
        lib().ish_o_matcher_batch(self._h, _ptr(recs, C.c_uint8), _ptr(offsets, C.c_uint64), n, threads,
                                  g("score", C.c_int32), g("qend", C.c_int32), g("tend", C.c_int32),
                                  g("hit", C.c_uint8), g("start", C.c_int64), g("end", C.c_int64))
        return {k: v[:n] for k, v in out.items()}

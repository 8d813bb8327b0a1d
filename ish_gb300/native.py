"""ctypes binding of libish_gpu.so (include/ish_gpu.h).

The library is built in-tree by ``ish_gb300.build``; loading fails loudly when
it is missing -- there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np


OK = 0
EINVAL, ENOMEM, EOVERFLOW, ENODEV, EDEVICE, EAGAIN, ETIMEDOUT = -22, -12, -75, -19, -5, -11, -110
ALGO_SEMI_GLOBAL, ALGO_LOCAL = 0, 1
FREE_QUERY_START, FREE_QUERY_END, FREE_TARGET_START, FREE_TARGET_END = 1, 2, 4, 8
KERNEL_AUTO, KERNEL_PLAIN, KERNEL_EXACT, KERNEL_PLAIN16 = 0, 1, 2, 3
OPT_KERNEL, OPT_SG_LANES, OPT_SW_U8_LANES, OPT_SW_U16_LANES, OPT_WAVE_GROUP, OPT_WAVE_K = 1, 2, 3, 4, 5, 6
OPT_PROFILE_LAYOUT = 7
OPT_WAVE_BLOCKS = 8
OPT_WAVE_LEAN = 9
OPT_WINDOWS = 10
OPT_STEP_BUDGET = 11
OPT_FAULT_ALLOC = 12
OPT_SERVE_STEP_CELLS = 13
PROF_AUTO, PROF_S16, PROF_PAIR, PROF_S32 = -1, 0, 1, 2

# Entry points declared in include/ish_gpu.h (checked by the tests).
EXPORTS = (
    "ish_gpu_abi_version", "ish_gpu_open", "ish_gpu_close", "ish_gpu_last_error", "ish_gpu_set_option",
    "ish_gpu_set_query", "ish_gpu_free_query", "ish_gpu_score", "ish_gpu_records_load", "ish_gpu_records_free",
    "ish_gpu_records_info", "ish_gpu_score_set", "ish_gpu_last_kernel_ms", "ish_gpu_calibrate",
    "ish_gpu_score_noalloc", "ish_gpu_score_multi", "ish_gpu_autotune", "ish_gpu_serve_start", "ish_gpu_submit",
    "ish_gpu_poll", "ish_gpu_serve_stop", "ish_gpu_serve_stats", "ish_gpu_match_starts",
    "ish_gpu_launch_count", "ish_gpu_records_load_raw", "ish_gpu_records_load_lines", "ish_gpu_last_windows",
    "ish_gpu_calibrate_lanes", "ish_gpu_records_load_fastx", "ish_gpu_records_get", "ish_gpu_last_load_ms",
    "ish_gpu_records_load_async",
)


class IshGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ish_gpu error {code}: {msg}")
        self.code = code


_lib = None

u8p = C.POINTER(C.c_uint8)
i8p = C.POINTER(C.c_int8)
i32p = C.POINTER(C.c_int32)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)


def lib_path() -> str:
    from . import build as _build

    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libish_gpu.so; raises if it is not built (or builds it on request)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build

    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is not built; run `python -m ish_gb300.build`")
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    L.ish_gpu_abi_version.restype = C.c_int
    L.ish_gpu_open.argtypes = [C.c_int, C.POINTER(vp)]
    L.ish_gpu_close.argtypes = [vp]
    L.ish_gpu_close.restype = None
    L.ish_gpu_last_error.argtypes = [vp]
    L.ish_gpu_last_error.restype = C.c_char_p
    L.ish_gpu_set_option.argtypes = [vp, C.c_int, C.c_int64]
    L.ish_gpu_set_query.argtypes = [vp, u8p, C.c_uint32, C.c_int, i8p, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32,
                                    C.c_uint32, C.c_int32, C.c_float, i32p]
    L.ish_gpu_free_query.argtypes = [vp, C.c_int32]
    L.ish_gpu_score.argtypes = [vp, C.c_int32, u8p, u64p, C.c_uint32, i32p, i32p, i32p, u8p, u32p, u32p]
    L.ish_gpu_records_load.argtypes = [vp, u8p, u64p, C.c_uint32, i32p]
    L.ish_gpu_records_load_async.argtypes = [vp, u8p, u64p, C.c_uint32, i32p]
    L.ish_gpu_records_free.argtypes = [vp, C.c_int32]
    L.ish_gpu_records_info.argtypes = [vp, C.c_int32, u32p, u64p]
    L.ish_gpu_score_set.argtypes = [vp, C.c_int32, C.c_int32, i32p, i32p, i32p, u8p, u32p, u32p]
    L.ish_gpu_last_kernel_ms.argtypes = [vp, C.POINTER(C.c_double)]
    L.ish_gpu_last_load_ms.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ish_gpu_calibrate.argtypes = [vp, C.POINTER(C.c_double)]
    L.ish_gpu_calibrate_lanes.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ish_gpu_score_noalloc.argtypes = [vp, C.c_uint64, vp, C.c_uint32, u8p, C.c_uint32, i8p, C.c_uint32, C.c_int,
                                        C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, C.c_float, vp, vp, vp, vp,
                                        vp, C.c_char_p, C.c_size_t]
    L.ish_gpu_score_multi.argtypes = [vp, i32p, C.c_uint32, C.c_int32, i32p, i32p, i32p, u8p, u32p, C.c_uint64, u64p]
    L.ish_gpu_autotune.argtypes = [vp, C.c_int32, i32p, C.c_uint32, i32p, i32p]
    L.ish_gpu_launch_count.argtypes = [vp, u64p]
    L.ish_gpu_last_windows.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.ish_gpu_records_load_raw.argtypes = [vp, u8p, u64p, C.c_uint32, C.c_int, i32p]
    L.ish_gpu_records_load_lines.argtypes = [vp, u8p, C.c_uint64, C.c_int, i32p, u32p]
    L.ish_gpu_records_load_fastx.argtypes = [vp, u8p, C.c_uint64, C.c_int, i32p, u32p, u64p, C.c_uint64]
    L.ish_gpu_records_get.argtypes = [vp, C.c_int32, C.c_uint32, C.c_uint32, u8p, C.c_uint64, u64p]
    L.ish_gpu_match_starts.argtypes = [vp, C.c_int32, C.c_int32, u32p, i32p, C.c_uint32, C.POINTER(C.c_int64)]
    L.ish_gpu_serve_start.argtypes = [vp, C.c_int32, C.c_uint32, C.c_uint64, C.c_uint32]
    L.ish_gpu_submit.argtypes = [vp, C.c_int32, u64p]
    L.ish_gpu_poll.argtypes = [vp, C.c_uint64, u32p, i32p, i32p, i32p, C.c_uint32, u32p, C.POINTER(C.c_double),
                               C.c_int32]
    L.ish_gpu_serve_stop.argtypes = [vp]
    L.ish_gpu_serve_stats.argtypes = [vp, u64p, C.POINTER(C.c_double), C.POINTER(C.c_double), u32p, u64p]
    for name in EXPORTS:
        if name not in ("ish_gpu_close", "ish_gpu_last_error"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def pack_records(records):
    """Concatenate a list of byte strings / uint8 arrays: (bytes uint8[], offsets uint64[n+1])."""
    lens = np.fromiter((len(r) for r in records), dtype=np.uint64, count=len(records))
    off = np.zeros(len(records) + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    buf = np.empty(int(off[-1]) if len(records) else 0, np.uint8)
    for i, r in enumerate(records):
        a, b = int(off[i]), int(off[i + 1])
        if b > a:
            buf[a:b] = np.frombuffer(r, np.uint8) if isinstance(r, (bytes, bytearray)) else r
    return buf, off


class Context:
    """One engine context on one CUDA device (one per host thread)."""

    def __init__(self, device: int = 0):
        L = load()
        h = C.c_void_p()
        rc = L.ish_gpu_open(device, C.byref(h))
        if rc != OK:
            raise IshGpuError(rc, L.ish_gpu_last_error(None).decode())
        self._L = L
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.ish_gpu_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise IshGpuError(rc, self._L.ish_gpu_last_error(self._h).decode())
        return rc

    def set_option(self, option: int, value: int):
        self._check(self._L.ish_gpu_set_option(self._h, option, int(value)))

    def set_query(self, enc_query, matrix_kind: int, matrix: np.ndarray, algo: int, gap_open: int, gap_ext: int,
                  ends_free: int, max_score: int, threshold: float) -> int:
        q = np.ascontiguousarray(enc_query, np.uint8)
        m = np.ascontiguousarray(matrix, np.int8).ravel()
        alphabet = int(round(len(m) ** 0.5))
        qid = C.c_int32()
        self._check(self._L.ish_gpu_set_query(self._h, _p(q, C.c_uint8), len(q), matrix_kind, _p(m, C.c_int8), alphabet,
                                              algo, gap_open, gap_ext, ends_free, int(max_score), float(threshold),
                                              C.byref(qid)))
        return qid.value

    def free_query(self, qid: int):
        self._check(self._L.ish_gpu_free_query(self._h, qid))

    def _outputs(self, n, want, out=None):
        """Output arrays for n records: the caller's (`out`, e.g. pinned host
        buffers reused across calls) where given and large enough, else new."""
        given = out or {}
        types = {"score": np.int32, "qend": np.int32, "tend": np.int32, "hit": np.uint8, "hit_idx": np.uint32}
        out = {}
        for k in want:
            a = given.get(k)
            if a is not None:
                if a.dtype != types[k] or len(a) < max(n, 1) or not a.flags.c_contiguous:
                    raise ValueError(f"output {k}: needs a contiguous {np.dtype(types[k])} array of {max(n, 1)}")
                out[k] = a
        if "score" in want and "score" not in out:
            out["score"] = np.empty(max(n, 1), np.int32)
        if "qend" in want and "qend" not in out:
            out["qend"] = np.empty(max(n, 1), np.int32)
        if "tend" in want and "tend" not in out:
            out["tend"] = np.empty(max(n, 1), np.int32)
        if "hit" in want and "hit" not in out:
            out["hit"] = np.empty(max(n, 1), np.uint8)
        if "hit_idx" in want and "hit_idx" not in out:
            out["hit_idx"] = np.empty(max(n, 1), np.uint32)
        return out

    def score(self, qid: int, records: np.ndarray, offsets: np.ndarray,
              want=("score", "qend", "tend", "hit", "hit_idx"), out=None) -> dict:
        """One-shot scoring of host records (ish_gpu_score): upload, pack,
        score, results back in one call.  `out` as for score_set."""
        records = np.ascontiguousarray(records, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        n = len(offsets) - 1
        out = self._outputs(n, want, out)
        nh = C.c_uint32()
        self._check(self._L.ish_gpu_score(self._h, qid, _p(records, C.c_uint8), _p(offsets, C.c_uint64), n,
                                          _p(out.get("score"), C.c_int32), _p(out.get("qend"), C.c_int32),
                                          _p(out.get("tend"), C.c_int32), _p(out.get("hit"), C.c_uint8),
                                          _p(out.get("hit_idx"), C.c_uint32), C.byref(nh)))
        res = {k: v[:n] for k, v in out.items() if k != "hit_idx"}
        if "hit_idx" in out:
            res["hit_idx"] = out["hit_idx"][: nh.value]
        return res

    def records_load(self, records: np.ndarray, offsets: np.ndarray) -> int:
        records = np.ascontiguousarray(records, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        sid = C.c_int32()
        self._check(self._L.ish_gpu_records_load(self._h, _p(records, C.c_uint8), _p(offsets, C.c_uint64),
                                                 len(offsets) - 1, C.byref(sid)))
        return sid.value

    def records_load_async(self, records: np.ndarray, offsets: np.ndarray) -> int:
        """Resident set whose upload and packing run on the load stream while
        the caller goes on (e.g. scores the previous set); the arrays are kept
        referenced here until the next load, since the copy may still read
        them."""
        records = np.ascontiguousarray(records, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        sid = C.c_int32()
        self._check(self._L.ish_gpu_records_load_async(self._h, _p(records, C.c_uint8), _p(offsets, C.c_uint64),
                                                       len(offsets) - 1, C.byref(sid)))
        self._inflight = (records, offsets)
        return sid.value

    def records_load_raw(self, raw: np.ndarray, offsets: np.ndarray, matrix_kind: int) -> int:
        """Resident set from raw bytes, encoded on the device for `matrix_kind`."""
        raw = np.ascontiguousarray(raw, np.uint8)
        offsets = np.ascontiguousarray(offsets, np.uint64)
        sid = C.c_int32()
        self._check(self._L.ish_gpu_records_load_raw(self._h, _p(raw, C.c_uint8), _p(offsets, C.c_uint64),
                                                     len(offsets) - 1, matrix_kind, C.byref(sid)))
        return sid.value

    def records_load_lines(self, text, matrix_kind: int):
        """Resident set of the lines of `text` (split and encoded on the device);
        returns (set id, number of lines)."""
        buf = np.frombuffer(bytes(text), np.uint8) if not isinstance(text, np.ndarray) else \
            np.ascontiguousarray(text, np.uint8)
        sid = C.c_int32()
        n = C.c_uint32()
        self._check(self._L.ish_gpu_records_load_lines(self._h, _p(buf, C.c_uint8) if len(buf) else None, len(buf),
                                                       matrix_kind, C.byref(sid), C.byref(n)))
        return sid.value, n.value

    def records_load_fastx(self, text, matrix_kind: int, bounds: bool = True):
        """Resident set of the FASTA/FASTQ records of `text` (split and encoded
        on the device as ish's FASTX runners read a file); returns (set id,
        number of records, bounds), bounds an (n, 4) uint64 array of name
        [start, end) and quality [start, end) byte offsets into `text` (None
        if not asked for)."""
        buf = np.frombuffer(bytes(text), np.uint8) if not isinstance(text, np.ndarray) else \
            np.ascontiguousarray(text, np.uint8)
        sid = C.c_int32()
        n = C.c_uint32()
        # every record needs a header line: at most one record per newline + 1
        cap = int(np.count_nonzero(buf == 10)) + 1 if bounds else 0
        bnd = np.zeros((cap, 4), np.uint64) if bounds else None
        self._check(self._L.ish_gpu_records_load_fastx(
            self._h, _p(buf, C.c_uint8) if len(buf) else None, len(buf), matrix_kind, C.byref(sid), C.byref(n),
            _p(bnd, C.c_uint64) if bounds else None, cap))
        return sid.value, n.value, (bnd[:n.value].copy() if bounds else None)

    def records_get(self, sid: int, first: int = 0, count: int | None = None):
        """Records [first, first + count) of a resident set, as stored
        (encoded), in record order: (codes, offsets)."""
        if count is None:
            count = self.records_info(sid)[0] - first
        off = np.zeros(count + 1, np.uint64)
        total = self.records_info(sid)[1]
        codes = np.zeros(max(1, int(total)), np.uint8)
        self._check(self._L.ish_gpu_records_get(self._h, sid, first, count, _p(codes, C.c_uint8), len(codes),
                                                _p(off, C.c_uint64)))
        return codes[:int(off[-1])], off

    def records_free(self, sid: int):
        self._check(self._L.ish_gpu_records_free(self._h, sid))

    def records_info(self, sid: int):
        n, b = C.c_uint32(), C.c_uint64()
        self._check(self._L.ish_gpu_records_info(self._h, sid, C.byref(n), C.byref(b)))
        return n.value, b.value

    def score_set(self, qid: int, sid: int, want=("score", "qend", "tend", "hit", "hit_idx"), out=None) -> dict:
        """Scores query `qid` against set `sid`.  `out` may hold the caller's
        output arrays (any of score/qend/tend/hit/hit_idx, at least n long);
        the results are views of them."""
        n, _ = self.records_info(sid)
        out = self._outputs(n, want, out)
        nh = C.c_uint32()
        self._check(self._L.ish_gpu_score_set(self._h, qid, sid, _p(out.get("score"), C.c_int32),
                                              _p(out.get("qend"), C.c_int32), _p(out.get("tend"), C.c_int32),
                                              _p(out.get("hit"), C.c_uint8), _p(out.get("hit_idx"), C.c_uint32),
                                              C.byref(nh)))
        res = {k: v[:n] for k, v in out.items() if k != "hit_idx"}
        if "hit_idx" in out:
            res["hit_idx"] = out["hit_idx"][: nh.value]
        return res

    def score_multi(self, qids, sid: int, want=("score", "qend", "tend", "hit", "hit_idx")) -> dict:
        """Batched launch of several queries against resident set `sid`.

        Arrays come back shaped (len(qids), n); "hit_idx" is a list with one
        array of ascending record indices per query."""
        n, _ = self.records_info(sid)
        q = np.ascontiguousarray(qids, np.int32)
        nq = len(q)
        tot = max(nq * n, 1)
        out = {}
        for k, dt in (("score", np.int32), ("qend", np.int32), ("tend", np.int32), ("hit", np.uint8)):
            if k in want:
                out[k] = np.empty(tot, dt)
        cap = 0
        idx = offs = None
        if "hit_idx" in want:
            cap = tot
            idx = np.empty(cap, np.uint32)
            offs = np.empty(nq + 1, np.uint64)
        self._check(self._L.ish_gpu_score_multi(
            self._h, _p(q, C.c_int32), nq, sid, _p(out.get("score"), C.c_int32), _p(out.get("qend"), C.c_int32),
            _p(out.get("tend"), C.c_int32), _p(out.get("hit"), C.c_uint8), _p(idx, C.c_uint32), cap,
            _p(offs, C.c_uint64)))
        res = {k: v[: nq * n].reshape(nq, n) for k, v in out.items()}
        if idx is not None:
            res["hit_idx"] = [idx[int(offs[i]):int(offs[i + 1])] for i in range(nq)]
        return res

    def autotune(self, sid: int, qids):
        """Times candidate kernel shapes for each query on a sample of set
        `sid`; returns the (group, cols) arrays now in use."""
        q = np.ascontiguousarray(qids, np.int32)
        g = np.zeros(max(len(q), 1), np.int32)
        k = np.zeros(max(len(q), 1), np.int32)
        self._check(self._L.ish_gpu_autotune(self._h, sid, _p(q, C.c_int32), len(q), _p(g, C.c_int32),
                                             _p(k, C.c_int32)))
        return g[: len(q)], k[: len(q)]

    def match_starts(self, qid: int, sid: int, hit_idx, target_end) -> np.ndarray:
        """Target starts of hits (device reverse pass): MatchResult(start, end + 1)."""
        h = np.ascontiguousarray(hit_idx, np.uint32)
        e = np.ascontiguousarray(target_end, np.int32)
        out = np.empty(max(len(h), 1), np.int64)
        self._check(self._L.ish_gpu_match_starts(self._h, qid, sid, _p(h, C.c_uint32), _p(e, C.c_int32), len(h),
                                                 _p(out, C.c_int64)))
        return out[: len(h)]

    # ---- serving loop ----
    def serve_start(self, sid: int, max_active: int = 64, mem_budget: int = 0, chunks: int = 8):
        self._check(self._L.ish_gpu_serve_start(self._h, sid, max_active, mem_budget, chunks))

    def submit(self, qid: int) -> int:
        t = C.c_uint64()
        self._check(self._L.ish_gpu_submit(self._h, qid, C.byref(t)))
        return t.value

    def poll(self, ticket: int, wait_ms: int = 0):
        """None while the query runs (after waiting up to wait_ms); else a dict
        with the hits -- record indices ("hit_idx") and their "score", "qend"
        and "tend" -- and "latency_ms" from submit to completion."""
        nh = C.c_uint32()
        lat = C.c_double()
        probe = np.zeros(1, np.uint32)
        # capacity 0: the call reports the hit count and keeps the result
        rc = self._L.ish_gpu_poll(self._h, ticket, _p(probe, C.c_uint32), None, None, None, 0, C.byref(nh),
                                  C.byref(lat), wait_ms)
        if rc == EAGAIN:
            return None
        k = nh.value
        out = {"hit_idx": np.empty(k, np.uint32), "score": np.empty(k, np.int32), "qend": np.empty(k, np.int32),
               "tend": np.empty(k, np.int32)}
        if rc == EOVERFLOW:
            rc = self._L.ish_gpu_poll(self._h, ticket, _p(out["hit_idx"], C.c_uint32), _p(out["score"], C.c_int32),
                                      _p(out["qend"], C.c_int32), _p(out["tend"], C.c_int32), k, C.byref(nh),
                                      C.byref(lat), 0)
        self._check(rc)
        out["latency_ms"] = lat.value
        return out

    def serve_stop(self):
        self._check(self._L.ish_gpu_serve_stop(self._h))

    def serve_stats(self) -> dict:
        done, steps = C.c_uint64(), C.c_uint64()
        cells, ms = C.c_double(), C.c_double()
        mx = C.c_uint32()
        self._check(self._L.ish_gpu_serve_stats(self._h, C.byref(done), C.byref(cells), C.byref(ms), C.byref(mx),
                                                C.byref(steps)))
        return {"completed": done.value, "cells": cells.value, "device_ms": ms.value, "max_active": mx.value,
                "steps": steps.value}

    def last_load_ms(self) -> dict:
        """Phases of the last record load: device upload (+ splitting),
        device packing, host wall time of the call (ms)."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self._check(self._L.ish_gpu_last_load_ms(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"upload": a.value, "pack": b.value, "wall": c.value}

    def calibrate(self) -> float:
        """Packed 16-bit DPX add-max instructions per second on this device."""
        r = C.c_double()
        self._check(self._L.ish_gpu_calibrate(self._h, C.byref(r)))
        return r.value

    def calibrate_lanes(self) -> dict:
        """Local-alignment cell updates per second on 2 x 16-bit (DPX) and
        4 x 8-bit (saturating SIMD byte) lanes, registers only."""
        a, b = C.c_double(), C.c_double()
        self._check(self._L.ish_gpu_calibrate_lanes(self._h, C.byref(a), C.byref(b)))
        return {"s16x2_cells_per_s": a.value, "u8x4_cells_per_s": b.value}

    def launch_count(self) -> int:
        """CUDA kernels the library has launched on this context."""
        c = C.c_uint64()
        self._check(self._L.ish_gpu_launch_count(self._h, C.byref(c)))
        return c.value

    def last_windows(self) -> int:
        """Windows the last single-query scoring call cut long records into (0: none)."""
        w = C.c_uint32()
        self._check(self._L.ish_gpu_last_windows(self._h, C.byref(w)))
        return w.value

    def last_kernel_ms(self) -> float:
        ms = C.c_double()
        self._check(self._L.ish_gpu_last_kernel_ms(self._h, C.byref(ms)))
        return ms.value

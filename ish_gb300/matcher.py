"""GPU matchers with the interface of ish's striped matchers.

``StripedSemiGlobalMatcher`` and ``StripedLocalMatcher`` mirror
ishlib/matcher/striped_semi_global_matcher.mojo:169-298 and
ishlib/matcher/striped_local_matcher.mojo:18-115 (constructor arguments,
pattern encoding, optimal score, threshold, the GpuMatcher accessors of
ishlib/matcher/__init__.mojo:79-121) and score whole batches of records on the
GB300 through libish_gpu.so: one call per batch in place of the per-record
``first_match`` of ishlib/cpu/process_batch.mojo:14-34.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import native
from .scoring import ScoringMatrix


@dataclass(frozen=True)
class SemiGlobalEndsFreeness:
    """--sg-ends-free (ishlib/searcher_settings.mojo:288-414)."""

    query_start: bool = False
    query_end: bool = False
    target_start: bool = True
    target_end: bool = True

    @staticmethod
    def from_str(value: str) -> "SemiGlobalEndsFreeness":
        if len(value) != 4:
            raise ValueError("Invalid SemiGlobalEndsFreeness specified. Must consist of 4 values like FFTT.")
        up = value.upper()
        if any(c not in "TF" for c in up):
            raise ValueError("Invalid SemiGlobalEndsFreeness specified. All values must be T or F")
        return SemiGlobalEndsFreeness(*(c == "T" for c in up))

    def mask(self) -> int:
        return ((native.FREE_QUERY_START if self.query_start else 0) | (native.FREE_QUERY_END if self.query_end else 0)
                | (native.FREE_TARGET_START if self.target_start else 0)
                | (native.FREE_TARGET_END if self.target_end else 0))


@dataclass
class BatchResult:
    """Per-record forward results and the match decisions of a batch."""

    score: np.ndarray       # int32: alignment score of the forward pass
    query_end: np.ndarray   # int32: 0-based inclusive
    target_end: np.ndarray  # int32: 0-based inclusive (-1: no alignment)
    hit: np.ndarray         # uint8: 1 iff the CPU matcher's first_match would match
    hit_idx: np.ndarray     # uint32: indices of the hits, ascending
    hit_start: np.ndarray | None = None  # int64 per hit: first_match's MatchResult.start (device reverse pass)

    def matches(self):
        """(record index, start, end) per hit: first_match's MatchResult(start, end)
        as ishlib/cpu/process_batch.mojo:56-66 builds it for GPU hits."""
        starts = self.hit_start if self.hit_start is not None else np.full(len(self.hit_idx), -1, np.int64)
        return [(int(i), int(s), int(self.target_end[i]) + 1) for i, s in zip(self.hit_idx, starts)]


class _GpuMatcherBase:
    algo = native.ALGO_SEMI_GLOBAL

    def __init__(self, pattern, score_threshold: float, matrix_kind="ascii", gap_open: int = 3,
                 gap_extend: int = 1, ends: int = 0, context: native.Context | None = None):
        self.matrix = ScoringMatrix.from_str(matrix_kind) if isinstance(matrix_kind, str) else ScoringMatrix(matrix_kind)
        self.pattern, self.max_score = self.matrix.encode_and_score(pattern)
        self.gap_open = int(gap_open)
        self.gap_extend = int(gap_extend)
        self._score_threshold = np.float32(score_threshold)
        self.ctx = context or native.Context(0)
        self.query_id = self.ctx.set_query(self.pattern, self.matrix.kind, self.matrix.values, self.algo,
                                           self.gap_open, self.gap_extend, ends, self.max_score,
                                           float(self._score_threshold))

    # Matcher / GpuMatcher accessors
    def encoded_pattern(self) -> np.ndarray:
        return self.pattern

    def max_alignment_score(self) -> int:
        return self.max_score

    def score_threshold(self) -> np.float32:
        return self._score_threshold

    def matrix_bytes(self) -> np.ndarray:
        return self.matrix.values.ravel()

    def matrix_len(self) -> int:
        return self.matrix.values.size

    def matrix_kind(self) -> int:
        return self.matrix.kind

    def convert_ascii_to_encoding(self, data) -> np.ndarray:
        return self.matrix.encode(data)

    def convert_encoding_to_ascii(self, codes) -> bytes:
        return self.matrix.decode(codes)

    # batch scoring on the GPU
    def batch_match(self, records, offsets=None, starts: bool = True) -> BatchResult:
        """Score encoded records: a list of arrays, or (concatenated bytes, offsets).
        With `starts`, the match start of every hit is found on the device too."""
        if offsets is None:
            records, offsets = native.pack_records(records)
        if not starts:
            r = self.ctx.score(self.query_id, records, offsets)
            return BatchResult(r["score"], r["qend"], r["tend"], r["hit"], r["hit_idx"])
        sid = self.ctx.records_load(records, offsets)
        try:
            return self.batch_match_resident(sid, starts=True)
        finally:
            self.ctx.records_free(sid)

    def batch_match_resident(self, set_id: int, starts: bool = True) -> BatchResult:
        r = self.ctx.score_set(self.query_id, set_id)
        hs = None
        if starts:
            hs = self.ctx.match_starts(self.query_id, set_id, r["hit_idx"], r["tend"][r["hit_idx"]])
        return BatchResult(r["score"], r["qend"], r["tend"], r["hit"], r["hit_idx"], hs)


class StripedSemiGlobalMatcher(_GpuMatcherBase):
    """GPU drop-in for StripedSemiGlobalMatcher (--match-algo striped-semi-global)."""

    algo = native.ALGO_SEMI_GLOBAL

    def __init__(self, pattern, score_threshold: float, sg_ends_free="FFTT", matrix_kind="ascii",
                 gap_open: int = 3, gap_extend: int = 1, context: native.Context | None = None):
        ends = sg_ends_free if isinstance(sg_ends_free, SemiGlobalEndsFreeness) else \
            SemiGlobalEndsFreeness.from_str(sg_ends_free)
        self.sg_ends_free = ends
        super().__init__(pattern, score_threshold, matrix_kind, gap_open, gap_extend, ends.mask(), context)


class StripedLocalMatcher(_GpuMatcherBase):
    """GPU drop-in for StripedLocalMatcher (--match-algo striped-local)."""

    algo = native.ALGO_LOCAL

    def __init__(self, pattern, score_threshold: float, matrix_kind="ascii", gap_open: int = 3,
                 gap_extend: int = 1, context: native.Context | None = None):
        super().__init__(pattern, score_threshold, matrix_kind, gap_open, gap_extend, 0, context)

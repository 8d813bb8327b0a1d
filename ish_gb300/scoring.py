"""Scoring matrices and encodings of ish, host side.

The tables restate ishlib/matcher/alignment/scoring_matrix.mojo:9-172 (same
values, same code order, as the records and queries handed to the GPU must be
encoded exactly like the reference encodes them) and the helpers restate
ScoringMatrix.convert_ascii_to_encoding_and_score (403-416) and
MatrixKind.from_str (185-196).
"""
from __future__ import annotations

import numpy as np

ASCII, ACTGN, ACTGN0, BLOSUM62 = 0, 1, 2, 3
KIND_NAMES = {"ascii": ASCII, "actgn": ACTGN, "actgn0": ACTGN0, "blosum62": BLOSUM62}

# Residue order of the BLOSUM62 table (scoring_matrix.mojo:30-35).
AA_ORDER = b"ARNDCQEGHILKMFPSTWYVBZX*"
_BLOSUM62_ROWS = """
 4 -1 -2 -2  0 -1 -1  0 -2 -1 -1 -1 -1 -2 -1  1  0 -3 -2  0 -2 -1  0 -4
-1  5  0 -2 -3  1  0 -2  0 -3 -2  2 -1 -3 -2 -1 -1 -3 -2 -3 -1  0 -1 -4
-2  0  6  1 -3  0  0  0  1 -3 -3  0 -2 -3 -2  1  0 -4 -2 -3  3  0 -1 -4
-2 -2  1  6 -3  0  2 -1 -1 -3 -4 -1 -3 -3 -1  0 -1 -4 -3 -3  4  1 -1 -4
 0 -3 -3 -3  9 -3 -4 -3 -3 -1 -1 -3 -1 -2 -3 -1 -1 -2 -2 -1 -3 -3 -2 -4
-1  1  0  0 -3  5  2 -2  0 -3 -2  1  0 -3 -1  0 -1 -2 -1 -2  0  3 -1 -4
-1  0  0  2 -4  2  5 -2  0 -3 -3  1 -2 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -2  0 -1 -3 -2 -2  6 -2 -4 -4 -2 -3 -3 -2  0 -2 -2 -3 -3 -1 -2 -1 -4
-2  0  1 -1 -3  0  0 -2  8 -3 -3 -1 -2 -1 -2 -1 -2 -2  2 -3  0  0 -1 -4
-1 -3 -3 -3 -1 -3 -3 -4 -3  4  2 -3  1  0 -3 -2 -1 -3 -1  3 -3 -3 -1 -4
-1 -2 -3 -4 -1 -2 -3 -4 -3  2  4 -2  2  0 -3 -2 -1 -2 -1  1 -4 -3 -1 -4
-1  2  0 -1 -3  1  1 -2 -1 -3 -2  5 -1 -3 -1  0 -1 -3 -2 -2  0  1 -1 -4
-1 -1 -2 -3 -1  0 -2 -3 -2  1  2 -1  5  0 -2 -1 -1 -1 -1  1 -3 -1 -1 -4
-2 -3 -3 -3 -2 -3 -3 -3 -1  0  0 -3  0  6 -4 -2 -2  1  3 -1 -3 -3 -1 -4
-1 -2 -2 -1 -3 -1 -1 -2 -2 -3 -3 -1 -2 -4  7 -1 -1 -4 -3 -2 -2 -1 -2 -4
 1 -1  1  0 -1  0  0  0 -1 -2 -2  0 -1 -2 -1  4  1 -3 -2 -2  0  0  0 -4
 0 -1  0 -1 -1 -1 -1 -2 -2 -1 -1 -1 -1 -2 -1  1  5 -2 -2  0 -1 -1  0 -4
-3 -3 -4 -4 -2 -2 -3 -2 -2 -3 -2 -3 -1  1 -4 -3 -2 11  2 -3 -4 -3 -2 -4
-2 -2 -2 -3 -2 -1 -2 -3  2 -1 -1 -2 -1  3 -3 -2 -2  2  7 -1 -3 -2 -1 -4
 0 -3 -3 -3 -1 -2 -2 -3 -3  3  1 -2  1 -1 -2 -2  0 -3 -1  4 -3 -2 -1 -4
-2 -1  3  4 -3  0  1 -1  0 -3 -4  0 -3 -3 -2  0 -1 -4 -3 -3  4  1 -1 -4
-1  0  0  1 -3  3  4 -2  0 -3 -3  1 -1 -3 -1  0 -1 -3 -2 -2  1  4 -1 -4
 0 -1 -1 -1 -2 -1 -1 -1 -1 -1 -1 -1 -1 -1 -2  0  0 -2 -1 -1 -1 -1 -1 -4
-4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4 -4  1
"""
NT_ORDER = b"ACGTN"


def _nt_table() -> np.ndarray:
    t = np.full(256, 4, np.uint8)
    for code, chars in enumerate((b"Aa", b"Cc", b"Gg", b"TtUu")):
        for c in chars:
            t[c] = code
    return t


def _aa_table() -> np.ndarray:
    t = np.full(256, 23, np.uint8)
    for code, c in enumerate(AA_ORDER):
        if 65 <= c <= 90:
            t[c] = code
            t[c + 32] = code
    return t


def _dna_matrix(n_score: int) -> np.ndarray:
    m = np.full((5, 5), -2, np.int8)
    np.fill_diagonal(m, 2)
    m[4, :] = n_score
    m[:, 4] = n_score
    return m


class ScoringMatrix:
    """Matrix values (row = record code, column = query code) plus encodings."""

    def __init__(self, kind: int):
        self.kind = kind
        if kind == ASCII:
            m = np.full((256, 256), -2, np.int8)
            np.fill_diagonal(m, 2)
            self.values = m
            self.ascii_to_code = np.arange(256, dtype=np.uint8)
            self.code_to_ascii = np.arange(256, dtype=np.uint8)
        elif kind in (ACTGN, ACTGN0):
            self.values = _dna_matrix(2 if kind == ACTGN else 0)
            self.ascii_to_code = _nt_table()
            self.code_to_ascii = np.frombuffer(NT_ORDER, np.uint8).copy()
        elif kind == BLOSUM62:
            self.values = np.array(_BLOSUM62_ROWS.split(), dtype=np.int8).reshape(24, 24)
            self.ascii_to_code = _aa_table()
            self.code_to_ascii = np.frombuffer(AA_ORDER, np.uint8).copy()
        else:
            raise ValueError(f"unknown matrix kind {kind}")
        self.size = self.values.shape[0]

    @staticmethod
    def from_str(name: str) -> "ScoringMatrix":
        try:
            return ScoringMatrix(KIND_NAMES[name.lower()])
        except KeyError:
            raise ValueError(f"Invalid scoring matrix name: {name}") from None

    def encode(self, data) -> np.ndarray:
        a = np.frombuffer(bytes(data), np.uint8) if not isinstance(data, np.ndarray) else data.astype(np.uint8, copy=False)
        return self.ascii_to_code[a]

    def decode(self, codes) -> bytes:
        return self.code_to_ascii[np.asarray(codes, np.uint8)].tobytes()

    def encode_and_score(self, data):
        """convert_ascii_to_encoding_and_score: (codes, optimal score)."""
        codes = self.encode(data)
        score = int(self.values[codes, codes].astype(np.int64).sum()) if len(codes) else 0
        return codes, score

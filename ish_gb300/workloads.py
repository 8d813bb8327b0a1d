"""Seeded synthetic workloads with the shapes of ish's benchmark configurations.

The reference benchmarks run on public data (UniProt Swiss-Prot queries and
targets, CHM13) that is not available here; these generators produce inputs
with the same sizes, length distributions and residue compositions, already
encoded with the matrix alphabet (what ish's runners hand to the matcher).

  line_ascii()     -- ascii line search, 24-byte query, 100,000 printable lines
  protein()        -- 300-residue query, 1,000,000 protein records
  nucleotide_multi() -- 64 queries x 2,000,000 short reads (batching pattern)
  long_targets()   -- 1,000-nt query, 10,000 records of 10 kb - 1 Mb
  serving_records() / serving_queries() -- resident protein set, Poisson stream
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .scoring import ACTGN, ACTGN0, ASCII, BLOSUM62, ScoringMatrix

# Background amino-acid frequencies of Robinson & Robinson (1991), in the
# residue order A R N D C Q E G H I L K M F P S T W Y V of the BLOSUM62 table
# (codes 0..19); these are the "standard background frequencies" used by
# BLAST's composition statistics.
AA_BACKGROUND = np.array([
    0.07805, 0.05129, 0.04487, 0.05364, 0.01925, 0.04264, 0.06295, 0.07377, 0.02199, 0.05142,
    0.09019, 0.05744, 0.02243, 0.03856, 0.05203, 0.07120, 0.05841, 0.01330, 0.03216, 0.06441,
])
AA_BACKGROUND = AA_BACKGROUND / AA_BACKGROUND.sum()


@dataclass
class Workload:
    name: str
    kind: int
    queries: list            # encoded queries (uint8 arrays)
    records: np.ndarray      # concatenated encoded records
    offsets: np.ndarray      # uint64[n+1]
    planted: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @property
    def lengths(self) -> np.ndarray:
        return np.diff(self.offsets).astype(np.int64)

    def cells(self, query_index: int | None = None) -> int:
        """Algorithmic cell updates: sum over queries of Q * sum of record lengths."""
        total = int(self.offsets[-1] - self.offsets[0])
        qs = self.queries if query_index is None else [self.queries[query_index]]
        return sum(len(q) for q in qs) * total

    def subset(self, idx: np.ndarray) -> "Workload":
        idx = np.asarray(idx, np.int64)
        lens = self.lengths[idx]
        off = np.zeros(len(idx) + 1, np.uint64)
        np.cumsum(lens, out=off[1:])
        buf = np.empty(int(off[-1]), np.uint8)
        starts = self.offsets[:-1][idx].astype(np.int64)
        for j, (s, l) in enumerate(zip(starts, lens)):
            buf[int(off[j]):int(off[j]) + l] = self.records[s:s + l]
        return Workload(self.name + "-subset", self.kind, self.queries, buf, off, meta=dict(self.meta))


_TABLES: dict = {}


def _table(probs):
    key = tuple(np.round(np.asarray(probs, np.float64), 12))
    t = _TABLES.get(key)
    if t is None:
        cdf = np.cumsum(probs)
        cdf[-1] = 1.0
        t = np.searchsorted(cdf, (np.arange(65536) + 0.5) / 65536.0).astype(np.uint8)
        _TABLES[key] = t
    return t


def _sample_codes(rng, n, probs=None, alphabet=None):
    """n i.i.d. codes; with `probs`, through a 65536-entry table (probabilities to 1/65536)."""
    if probs is None:
        return rng.integers(0, alphabet, n, dtype=np.uint8)
    return _table(probs)[rng.integers(0, 65536, n, dtype=np.uint16)]


def _offsets(lens):
    off = np.zeros(len(lens) + 1, np.uint64)
    np.cumsum(np.asarray(lens, np.uint64), out=off[1:])
    return off


def _mutate(rng, q, sub_rate, indel_rate, alphabet_sampler):
    """Copy of q with substitutions and single-residue insertions/deletions."""
    out = []
    for c in q:
        r = rng.random()
        if r < indel_rate / 2:          # deletion
            continue
        if r < indel_rate:              # insertion before this residue
            out.append(int(alphabet_sampler(1)[0]))
        out.append(int(alphabet_sampler(1)[0]) if rng.random() < sub_rate else int(c))
    return np.array(out, np.uint8)


def _plant(rng, records, off, which, make_copy):
    """Overwrite a window of each chosen record with a mutated query copy."""
    for i in which:
        a, b = int(off[i]), int(off[i + 1])
        cp = make_copy()
        L = b - a
        if len(cp) > L:
            cp = cp[:L]
        pos = int(rng.integers(0, L - len(cp) + 1))
        records[a + pos:a + pos + len(cp)] = cp


def line_ascii(seed: int = 0, n: int = 100_000, qlen: int = 24, planted_frac: float = 0.01) -> Workload:
    """Plain semi-global line search: ascii (+2/-2), printable query and lines (0x20-0x7E)."""
    rng = np.random.default_rng(seed)
    q = rng.integers(0x20, 0x7F, qlen, dtype=np.uint8)
    lens = rng.integers(20, 121, n)
    off = _offsets(lens)
    recs = rng.integers(0x20, 0x7F, int(off[-1]), dtype=np.uint8)
    which = np.sort(rng.choice(n, int(round(n * planted_frac)), replace=False))
    samp = lambda k: rng.integers(0x20, 0x7F, k, dtype=np.uint8)
    _plant(rng, recs, off, which, lambda: _mutate(rng, q, 0.10, 0.02, samp))
    return Workload("line-ascii", ASCII, [q], recs, off, which,
                    dict(gap_open=3, gap_extend=1, ends="FFTT", threshold=0.8, algo="striped-semi-global"))


def protein(seed: int = 1, n: int = 1_000_000, qlen: int = 300, planted_frac: float = 0.001,
            median: float = 350.0, sigma: float = 0.6, lo: int = 30, hi: int = 5000) -> Workload:
    """Single-query protein search: blosum62, log-normal record lengths, 0.1% planted at 40% substitution."""
    rng = np.random.default_rng(seed)
    q = _sample_codes(rng, qlen, AA_BACKGROUND)
    lens = np.clip(np.round(rng.lognormal(np.log(median), sigma, n)), lo, hi).astype(np.int64)
    off = _offsets(lens)
    recs = _sample_codes(rng, int(off[-1]), AA_BACKGROUND)
    which = np.sort(rng.choice(n, max(1, int(round(n * planted_frac))), replace=False))
    samp = lambda k: _sample_codes(rng, k, AA_BACKGROUND)
    _plant(rng, recs, off, which, lambda: _mutate(rng, q, 0.40, 0.0, samp))
    return Workload("protein", BLOSUM62, [q], recs, off, which,
                    dict(gap_open=10, gap_extend=1, ends="FFTT", threshold=0.8))


def _nucleotides(rng, n, gc=0.5, n_rate=0.005):
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]) * (1 - n_rate)
    return _sample_codes(rng, n, np.append(p, n_rate))


def nucleotide_multi(seed: int = 2, nq: int = 64, n: int = 2_000_000, qmin: int = 50, qmax: int = 1000,
                     rmin: int = 100, rmax: int = 300) -> Workload:
    """Batched multi-query nucleotide search: actgn, 0.5% N in queries and reads."""
    rng = np.random.default_rng(seed)
    qs = [_nucleotides(rng, int(L)) for L in rng.integers(qmin, qmax + 1, nq)]
    lens = rng.integers(rmin, rmax + 1, n)
    off = _offsets(lens)
    recs = _nucleotides(rng, int(off[-1]))
    return Workload("nucleotide-multi", ACTGN, qs, recs, off,
                    meta=dict(gap_open=3, gap_extend=1, ends="FFTT", threshold=0.8))


def long_targets(seed: int = 3, n: int = 10_000, qlen: int = 1000, lmin: float = 1e4, lmax: float = 1e6,
                 planted: int = 50) -> Workload:
    """Long-target semi-global: actgn0, log-uniform record lengths, GC 40%, 0.5% N, planted copies at 5%."""
    rng = np.random.default_rng(seed)
    q = _nucleotides(rng, qlen, gc=0.4)
    lens = np.round(np.exp(rng.uniform(np.log(lmin), np.log(lmax), n))).astype(np.int64)
    off = _offsets(lens)
    recs = _nucleotides(rng, int(off[-1]), gc=0.4)
    which = np.sort(rng.choice(n, min(planted, n), replace=False))
    samp = lambda k: _nucleotides(rng, k, gc=0.4)
    _plant(rng, recs, off, which, lambda: _mutate(rng, q, 0.05, 0.0, samp))
    return Workload("long-targets", ACTGN0, [q], recs, off, which,
                    meta=dict(gap_open=3, gap_extend=1, ends="FFTT", threshold=0.8))


def serving_records(seed: int = 4, total_bytes: int = 4 << 30, median: float = 350.0, sigma: float = 0.6) -> Workload:
    """Resident protein set for the serving loop (blosum62 codes, log-normal lengths)."""
    rng = np.random.default_rng(seed)
    mean = median * np.exp(sigma * sigma / 2)
    n = int(total_bytes / mean)
    lens = np.clip(np.round(rng.lognormal(np.log(median), sigma, n)), 30, 5000).astype(np.int64)
    off = _offsets(lens)
    recs = _sample_codes(rng, int(off[-1]), AA_BACKGROUND)
    return Workload("serving", BLOSUM62, [], recs, off, meta=dict(gap_open=10, gap_extend=1))


def serving_queries(seed: int = 5, count: int = 64, qmin: int = 20, qmax: int = 2000, rate: float = 10.0):
    """Poisson arrival stream: list of (arrival_s, algo, encoded query)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        L = int(rng.integers(qmin, qmax + 1))
        algo = "striped-local" if rng.random() < 0.5 else "striped-semi-global"
        out.append((float(t[i]), algo, _sample_codes(rng, L, AA_BACKGROUND)))
    return out


def matrix_for(kind: int) -> ScoringMatrix:
    return ScoringMatrix(kind)

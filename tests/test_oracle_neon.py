"""The oracle's NEON vector passes against its lane loops.

On an aarch64 host the oracle runs the striped passes at the reference's own
lane counts on NEON vectors (oracle/ish_oracle_neon.c), as ish runs them on
Grace; elsewhere it has only the lane loops.  The aarch64 host of this
project is the GPU machine, so the test carries the gpu marker to run there (it
uses no GPU) and skips where the vector passes are not built.  Every score,
end coordinate, hit and match start must be identical both ways.
"""
import numpy as np
import pytest

import oracle as O
from ish_gb300.scoring import ScoringMatrix

pytestmark = pytest.mark.gpu


def _batch(m, buf, off):
    return m.batch(buf, off, threads=4, forward=True, matches=True)


@pytest.mark.skipif(not O.lib() or not O.lib().ish_o_neon_available(), reason="no NEON vector passes on this host")
@pytest.mark.parametrize("kind", [O.BLOSUM62, O.ACTGN, O.ASCII])
def test_vector_passes_equal_lane_loops(kind):
    rng = np.random.default_rng(83 + kind)
    sm = ScoringMatrix(kind)
    alpha = {O.BLOSUM62: 20, O.ACTGN: 5, O.ASCII: 4}[kind]
    for trial in range(24):
        Q = int(rng.integers(1, 400))
        q = rng.integers(0, alpha, Q, dtype=np.uint8)
        if kind == O.ASCII:
            q = q + ord("a")
        recs = []
        for _ in range(60):
            r = rng.integers(0, alpha, int(rng.integers(0, 700)), dtype=np.uint8)
            if kind == O.ASCII:
                r = r + ord("a")
            if rng.random() < 0.2 and len(r) > Q:
                pos = int(rng.integers(0, len(r) - Q + 1))
                r[pos:pos + Q] = q
            recs.append(r)
        lens = np.array([len(r) for r in recs], np.uint64)
        off = np.zeros(len(recs) + 1, np.uint64)
        np.cumsum(lens, out=off[1:])
        buf = np.concatenate(recs) if int(off[-1]) else np.zeros(0, np.uint8)
        mx = int(sm.values[q, q].astype(np.int64).sum())
        gaps = [(10, 1), (3, 1), (5, 2), (1, 1)][trial % 4]
        for algo, ends in ((O.SEMI_GLOBAL, trial % 16), (O.LOCAL, 0)):
            m = O.Matcher(algo, kind, q, mx, 0.5, gap_open=gaps[0], gap_extend=gaps[1], ends=ends)
            O.set_vectors(True)
            assert O.vectors()
            v = _batch(m, buf, off)
            O.set_vectors(False)
            s = _batch(m, buf, off)
            O.set_vectors(True)
            for k in v:
                assert np.array_equal(v[k], s[k]), (kind, trial, algo, ends, k)

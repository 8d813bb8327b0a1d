"""End-to-end match sets of ish's own searcher test, through the CPU oracle.

tests/test_searcher.mojo:131-200 runs do_search for striped-local and
striped-semi-global (ends TTTT and FFTT) with threshold 0.8, gap 3/1, and
expects the same output for every combination.  The oracle's matchers must
reproduce those outputs exactly (fastx compared upper-cased, as at 186-187).
"""
import numpy as np
import pytest

import oracle as O
from searcher_fixtures import cases, records, render

SETTINGS = [(O.LOCAL, "FFTT"), (O.SEMI_GLOBAL, "TTTT"), (O.SEMI_GLOBAL, "FFTT")]


@pytest.mark.parametrize("case", cases(), ids=lambda c: f"{c['matrix']}-{c['record_type']}-{c['line']}")
@pytest.mark.parametrize("algo,ends", SETTINGS)
def test_searcher_case(case, algo, ends):
    kind = O.MATRIX_NAMES[case["matrix"]]
    _, _, _, c2a = O.matrix(kind)
    m = O.Matcher.from_ascii(algo, kind, case["pattern"].encode(), 0.8, gap_open=3, gap_extend=1,
                             ends=O.ends_from_str(ends))
    recs = records(case)
    encoded = [O.encode(kind, seq) for _, seq in recs]
    hits = [m.first_match(e) is not None for e in encoded]
    got = render(case, recs, hits, c2a, encoded)
    if case["record_type"] == "fastx":
        assert got.upper() == case["expected"].upper()
    else:
        assert got == case["expected"]

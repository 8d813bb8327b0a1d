"""Regenerate the golden fixtures in this folder from the ish reference tests.

Run inside a checkout that has the ish sources next to it:

    python tests/golden/make_golden.py /path/to/ish

The reference is written in Mojo and cannot be executed here, so the fixtures
are the inputs its own tests feed the aligners, read from the test files as
text: every string literal of every test function (in source order), plus the
four end-to-end search fixtures of tests/test_searcher.mojo:17-128 with their
expected match output.  The expected scores and coordinates those tests assert
are restated, with file:line citations, in tests/test_oracle_kat.py.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _fn_bodies(src: str):
    """Yield (name, first_line, body) for every top-level `fn`/`def`."""
    heads = [(m.group(2), m.start()) for m in re.finditer(r"^(fn|def) (\w+)", src, re.M)]
    for i, (name, pos) in enumerate(heads):
        end = heads[i + 1][1] if i + 1 < len(heads) else len(src)
        yield name, src.count("\n", 0, pos) + 1, src[pos:end]


def _literals(body: str):
    # "..." string literals, skipping the triple-quoted docstrings.
    body = re.sub(r'"""[\s\S]*?"""', "", body)
    out = []
    for m in re.finditer(r'"((?:[^"\\\n]|\\.)*)"\s*\.as_bytes\(\)', body):
        out.append(m.group(1))
    return out


def extract_literals(path: str):
    src = open(path, encoding="utf-8").read()
    return {name: {"line": line, "bytes": _literals(body)} for name, line, body in _fn_bodies(src)}


def extract_searcher_cases(path: str):
    src = open(path, encoding="utf-8").read()
    aliases = {m.group(1): m.group(2) for m in re.finditer(r'alias (\w+) = """([\s\S]*?)"""', src)}
    cases = []
    for m in re.finditer(r"TestCase\(\s*in_data=(\w+),\s*pattern=List\(\s*\"([^\"]*)\"\s*\.as_bytes\(\)\s*\),"
                         r"\s*expected=\"\"\"([\s\S]*?)\"\"\",\s*matrix_kind=MatrixKind\.(\w+),"
                         r"\s*record_type=\"(\w+)\"", src):
        cases.append({
            "line": src.count("\n", 0, m.start()) + 1,
            "in_data": aliases[m.group(1)],
            "pattern": m.group(2),
            "expected": m.group(3),
            "matrix": m.group(4).lower(),
            "record_type": m.group(5),
        })
    return cases


def main(ref_root: str):
    tests = os.path.join(ref_root, "tests")
    out = {
        "source": "ish v1.4.0 tests (Mojo), extracted as text by tests/golden/make_golden.py",
        "test_semi_global.mojo": extract_literals(os.path.join(tests, "test_semi_global.mojo")),
        "test_local_and_profile.mojo": extract_literals(os.path.join(tests, "test_local_and_profile.mojo")),
    }
    with open(os.path.join(HERE, "kat_inputs.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    cases = extract_searcher_cases(os.path.join(tests, "test_searcher.mojo"))
    assert len(cases) == 5, len(cases)
    with open(os.path.join(HERE, "searcher_cases.json"), "w") as f:
        json.dump({"source": "ish v1.4.0 tests/test_searcher.mojo (settings loop at 131-171)",
                   "cases": cases}, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

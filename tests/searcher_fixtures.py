"""Record parsing and output formatting for the end-to-end searcher fixtures.

Mirrors what ish's parallel runners do with a file before and after matching:
line records split on '\\n' with '\\r' stripped (ishlib/vendor/kseq.mojo:270-330),
FASTA records as header + concatenated sequence lines
(ishlib/vendor/kseq.mojo:370-461), and matched records printed decoded
(ishlib/parallel_line_search_runner.mojo:113-155,
ishlib/parallel_fastx_search_runner.mojo:136-177).
"""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    return json.load(open(os.path.join(HERE, "golden", "searcher_cases.json")))["cases"]


def kseq_lines(data: bytes):
    """Lines as ish's reader returns them (ishlib/vendor/kseq.mojo:270-330,
    read_until with the newline delimiter): split at '\\n'; a trailing '\\r' is
    dropped from a line longer than one byte; a last line without '\\n' is a
    record; a final '\\n' does not start another one."""
    out, pos, n = [], 0, len(data)
    while pos < n:
        r = data.find(b"\n", pos)
        line = data[pos:] if r < 0 else data[pos:r]
        pos = n if r < 0 else r + 1
        if len(line) > 1 and line[-1] == 13:
            line = line[:-1]
        out.append(line)
    return out


def line_records(text: str):
    return [(None, line) for line in kseq_lines(text.encode())]


def fasta_records(text: str):
    """(name, sequence) of every record, through the oracle's restatement of
    ish's FASTX reader (ishlib/vendor/kseq.mojo:370-461)."""
    from oracle.fastx import read_records

    return [(name, seq) for name, seq, _ in read_records(text.encode())]


def records(case):
    return line_records(case["in_data"]) if case["record_type"] == "line" else fasta_records(case["in_data"])


def render(case, recs, hits, code_to_ascii, encoded):
    """Output text of the runner for these hits, through the library's own
    writer (ish_gb300.output): matched records, decoded, in input order."""
    import numpy as np

    from ish_gb300 import output

    enc = [np.asarray(e, np.uint8) for e in encoded]
    off = np.zeros(len(enc) + 1, np.uint64)
    np.cumsum([len(e) for e in enc], out=off[1:])
    buf = np.concatenate(enc) if enc else np.zeros(0, np.uint8)
    matches = [(i, 0, 0) for i, h in enumerate(hits) if h]
    c2a = np.asarray(code_to_ascii, np.uint8)
    parts = []
    if case["record_type"] == "line":
        output.write_line_matches(parts.append, buf, off, matches, c2a)
    else:
        output.write_fastx_matches(parts.append, [h for h, _ in recs], buf, off, matches, c2a)
    return b"".join(parts).decode("utf-8", errors="surrogateescape")

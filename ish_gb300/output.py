"""Matched records written the way ish's parallel runners write them.

The runners print every matched record DECODED (codes back to ascii through
the matrix's code table, so actgn input comes out upper case with every
non-ACGT byte as N), in input order, one result per record:

  line records   ishlib/parallel_line_search_runner.mojo:113-155
                 plain: the decoded line + "\\n"; on a tty:
                 PURPLE file RESET ":" GREEN line_number RESET ": " then the
                 line with the match [start, end) in RED ... RESET
  fastx records  ishlib/parallel_fastx_search_runner.mojo:136-177
                 ">" name "\\n", the decoded sequence (on a tty the match in
                 "\\033[1;31m" RED ... RESET), for FASTQ "\\n+\\n" quality, "\\n"

`matches` are (record index, start, end) triples with an exclusive end, as
``BatchResult.matches()`` and the runners' MatchResult give them, ascending by
record index.  `write` receives bytes (e.g. ``sys.stdout.buffer.write``).
"""
from __future__ import annotations

import numpy as np

RED = b"\x1b[31m"
GREEN = b"\x1b[32m"
PURPLE = b"\x1b[35m"
RESET = b"\x1b[0m"
BOLD_RED = b"\x1b[1;31m"


def _decoded(code_to_ascii: np.ndarray, records: np.ndarray, offsets: np.ndarray, i: int) -> bytes:
    a, b = int(offsets[i]), int(offsets[i + 1])
    return code_to_ascii[records[a:b]].tobytes() if b > a else b""


def write_line_matches(write, records, offsets, matches, code_to_ascii, file_name: bytes = b"",
                       first_line: int = 0, tty: bool = False) -> None:
    """Line runner output for encoded line records (`records[offsets[i]:offsets[i+1]]`);
    `first_line` is the number of lines of the file before this batch."""
    for i, s, e in matches:
        line = _decoded(code_to_ascii, records, offsets, i)
        if tty:
            write(PURPLE + file_name + RESET + b":" + GREEN + str(int(i) + first_line + 1).encode() + RESET + b": "
                  + line[0:s] + RED + line[s:e] + RESET + line[e:] + b"\n")
        else:
            write(line + b"\n")


def write_fastx_matches(write, names, records, offsets, matches, code_to_ascii, quals=None,
                        tty: bool = False) -> None:
    """FASTA/FASTQ runner output: `names[i]` is record i's header line without
    its '>'/'@', `quals[i]` its FASTQ quality line (None for FASTA)."""
    for i, s, e in matches:
        seq = _decoded(code_to_ascii, records, offsets, i)
        out = b">" + bytes(names[i]) + b"\n"
        out += (seq[0:s] + BOLD_RED + RED + seq[s:e] + RESET + seq[e:]) if tty else seq
        if quals is not None:
            out += b"\n+\n" + bytes(quals[i])
        write(out + b"\n")

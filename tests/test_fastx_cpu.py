"""The device FASTA/FASTQ splitter's line machine, modelled on the CPU and
checked against the oracle's byte-level restatement of ish's reader.

ish_gb300/csrc/fastx.cu decides every line's role from the reader's state at
the line start (SEEK, SEQ, ABS, QUAL) and gets those states from a prefix scan
of per-line state maps.  `line_machine` below is the same computation written
sequentially: the same per-line map, the same roles, byte counts and record
checks.  On random texts built from the bytes that matter to the reader
('>', '@', '+', '\\r', '\\n' among ordinary ones) it must give exactly the
records of oracle.fastx.read_records (ishlib/vendor/kseq.mojo:370-461), or
refuse exactly when the reader would go on to a second quality line.
"""
import numpy as np

from oracle.fastx import read_records

SEEK, SEQ, ABS, QUAL = 0, 1, 2, 3


def lines_of(data: bytes):
    """(start, end, has_newline) of every line: split at '\\n', a last line
    without '\\n' counts, a final '\\n' starts no line."""
    out, pos, n = [], 0, len(data)
    while pos < n:
        r = data.find(b"\n", pos)
        if r < 0:
            out.append((pos, n, False))
            break
        out.append((pos, r, True))
        pos = r + 1
    return out


def seq_char(data, s, e, nl):
    k = s
    while k < e and data[k] == 13:
        k += 1
    return k, (data[k] if k < e else (10 if nl else -1))


def line_map(data, s, e, nl):
    hc = min([data.find(b">", s, e), data.find(b"@", s, e)], key=lambda x: x if x >= 0 else 1 << 62)
    _, c = seq_char(data, s, e, nl)
    on_seek = SEQ if hc >= 0 else SEEK
    on_seq = QUAL if c == ord("+") else (ABS if c == 10 else SEQ)
    return (on_seek, on_seq, SEQ, SEEK), hc


def line_machine(data: bytes):
    """Records (name, seq, qual-or-None) as the device splits them, or the
    string 'continued' where the device refuses the file."""
    L = lines_of(data)
    n = len(L)
    st = SEEK
    recs = []  # dicts: name bounds, seq parts, flags
    for i, (s, e, nl) in enumerate(L):
        m, hc = line_map(data, s, e, nl)
        if st == SEEK:
            if hc >= 0:
                recs.append({"h": hc, "e": e, "seq": [], "plus": False, "qual": None, "more": False, "stop": False})
        elif st == SEQ:
            sp, c = seq_char(data, s, e, nl)
            if c < 0:
                pass
            elif c == 10:
                recs[-1]["seq"].append(b"\n")
            elif c in (ord(">"), ord("@")):
                recs.append({"h": sp, "e": e, "seq": [], "plus": False, "qual": None, "more": False, "stop": False})
            elif c == ord("+"):
                recs[-1]["plus"] = True
                if not nl or i + 1 >= n:
                    recs[-1]["stop"] = True
            else:
                part = data[sp:e]
                if len(part) > 1 and part[-1] == 13:
                    part = part[:-1]
                recs[-1]["seq"].append(part)
        elif st == ABS:
            part = data[s:e]
            if len(part) >= 1 and part[-1] == 13:
                part = part[:-1]
            recs[-1]["seq"].append(part)
        else:
            q = data[s:e]
            if len(q) > 1 and q[-1] == 13:
                q = q[:-1]
            recs[-1]["qual"] = q
            recs[-1]["more"] = i + 1 < n
        st = m[st]
    out = []
    for r in recs:
        name = data[r["h"] + 1:r["e"]]
        if len(name) > 1 and name[-1] == 13:
            name = name[:-1]
        seq = b"".join(r["seq"])
        stop = r["stop"] or len(seq) == 0 or r["h"] + 1 >= len(data)
        if not stop and r["plus"]:
            q = r["qual"]
            if q is None or len(q) > len(seq):
                stop = True
            elif len(q) < len(seq):
                if r["more"]:
                    return "continued"
                stop = True
        if stop:
            break
        out.append((name, seq, r["qual"] if r["plus"] else None))
    return out


def random_text(rng, n_tokens):
    """Texts from record-shaped fragments and the reader's special bytes."""
    frags = [b">", b"@", b"+", b"\n", b"\r", b"\r\n", b"ACGT", b"N", b"x y", b"II", b"I", b"@I", b">a\n", b"@r\n",
             b"AC\n+\nII\n", b"ACG\n", b"\n\n", b" ", b"+x\n"]
    idx = rng.integers(0, len(frags), n_tokens)
    return b"".join(frags[i] for i in idx)


def expected(data):
    recs, continued = read_records(data, with_continued=True)
    return "continued" if continued else recs


def test_line_machine_on_handwritten_files():
    cases = [
        b">a x\nACGT\nAC\r\n>b\nGG\n",  # multi-line, CRLF
        b"@r1\nACGT\n+\n@III\n@r2\nAC\n+r2\nII\n",  # a quality line that starts with '@'
        b"junk>h1\nAC\n>h2\nTT",  # text before the first header, header mid-line, no final newline
        b">a\nAC\n\n>b\nGG\n",  # an empty line swallows the next header
        b">a\nAC\n>b\n>c\nT\n",  # an empty record ends the file
        b"@r1\nAC\n+\nIII\n@r2\nA\n+\nI\n",  # quality longer than the sequence ends the file
        b"@r1\nACGT\n+\nII\nII\n",  # a continued quality
        b"@r1\nAC\n+\n",  # no quality line
        b">a\nAC\n>",  # a header byte at the end of the file
        b"\r\r>a\r\n\rAC\r\n\r\n",  # carriage returns everywhere
        b">a\nAC\n@q\nGT\n+\nII\n>c\nA\n",  # FASTA and FASTQ mixed
        b"", b"\n\n\n", b"no header at all\n",
    ]
    for data in cases:
        assert line_machine(data) == expected(data), data


def test_line_machine_on_random_texts():
    rng = np.random.default_rng(2024)
    for trial in range(3000):
        data = random_text(rng, int(rng.integers(1, 40)))
        assert line_machine(data) == expected(data), data

"""CPU restatement of ish's FASTA/FASTQ record reader.

TEST INFRASTRUCTURE ONLY: the parity checker for the device-side FASTA/FASTQ
splitter (``ish_gpu_records_load_fastx``).  Nothing in the product imports it.

It follows, byte by byte, ``FastxReader[read_comment=False].read`` of
ishlib/vendor/kseq.mojo:370-461 over ``BufferedReader.read_byte`` (248-262)
and ``read_until`` (270-324), and the loop of the FASTX runners that calls it
(ishlib/parallel_fastx_search_runner.mojo:93-121 and 339-362): records are
read until the first call that returns 0 or less (end of file, an empty
sequence, a FASTQ quality of the wrong length or a missing quality line).
"""
from __future__ import annotations

NL, CR, FA, FQ, PLUS = 10, 13, ord(">"), ord("@"), ord("+")


class _Reader:
    """The reference's buffered reader over an in-memory file.  Its refills
    are invisible at this level: read_until keeps appending across them."""

    def __init__(self, data: bytes):
        self.d = data
        self.i = 0

    def read_byte(self) -> int:  # kseq.mojo:248-262
        if self.i >= len(self.d):
            return -1
        c = self.d[self.i]
        self.i += 1
        return c

    def read_until_newline(self, buf: bytearray, offset: int) -> int:  # kseq.mojo:270-324
        del buf[offset:]
        if self.i >= len(self.d):
            return -1  # nothing read and end of file
        r = self.d.find(b"\n", self.i)
        if r < 0:
            r = len(self.d)
        buf += self.d[self.i:r]
        self.i = r + 1
        if len(buf) > 1 and buf[-1] == CR:  # "Handle \r": the whole buffer's last byte
            del buf[-1]
        return len(buf)


class FastxReader:
    """kseq.mojo:335-461 with read_comment=False (the runners' setting)."""

    def __init__(self, data: bytes):
        self.r = _Reader(data)
        self.name = bytearray()
        self.seq = bytearray()
        self.qual = bytearray()
        self.last_char = 0
        self.fastq = False
        self.qual_lines = 1
        # byte offsets of the last record's header line (after the '>'/'@')
        # and quality line, for the device loader's bounds
        self.name_start = 0
        self.qual_start = 0

    def read(self) -> int:
        r = self.r
        if self.last_char == 0:  # 383-393: seek the next header character
            c = r.read_byte()
            while c >= 0 and c != FA and c != FQ:
                c = r.read_byte()
            if c < 0:
                return c
        self.seq.clear()
        self.qual.clear()
        self.name.clear()
        self.fastq = False
        self.qual_lines = 1  # quality lines read (more than one: a continued quality)
        self.name_start = r.i
        if r.read_until_newline(self.name, 0) < 0:  # 416-421
            return -1
        c = r.read_byte()  # 423-440: sequence lines
        while c >= 0 and c != FA and c != PLUS and c != FQ:
            if c == CR:  # 429-431: a '\r' is skipped, the next byte is tested
                c = r.read_byte()
                continue
            self.seq.append(c)
            r.read_until_newline(self.seq, len(self.seq))
            c = r.read_byte()
        if c == FA or c == FQ:
            self.last_char = c
        if c != PLUS:
            return len(self.seq)
        c = r.read_byte()  # 445-451: the rest of the '+' line
        while c >= 0 and c != NL:
            c = r.read_byte()
        if c < 0:
            return -2
        self.qual_start = r.i
        rr = r.read_until_newline(self.qual, len(self.qual))  # 454-461
        while rr >= 0 and len(self.qual) < len(self.seq):
            rr = r.read_until_newline(self.qual, len(self.qual))
            if rr >= 0:
                self.qual_lines += 1
        if rr < 0:
            return -3
        self.last_char = 0
        if len(self.qual) != len(self.seq):
            return -2
        self.fastq = True
        return len(self.seq)


def read_records(data: bytes, with_continued=False):
    """The records a FASTX runner takes from a file: a list of
    (name, seq, qual-or-None), stopping at the first read() <= 0.  With
    `with_continued`, also whether the reader went past a record's first
    quality line before it stopped (a quality continued on the next line)."""
    rd = FastxReader(data)
    out = []
    continued = False
    while True:
        rd.qual_lines = 1
        ret = rd.read()
        continued = continued or rd.qual_lines > 1
        if ret <= 0:
            return (out, continued) if with_continued else out
        out.append((bytes(rd.name), bytes(rd.seq), bytes(rd.qual) if rd.fastq else None))

"""FASTA ingest, as ReadFasta.read (phylogenetics_analysis/ReadFasta.java:8-46)
and SequenceAnalysisContext.parseFiles (:60-76).

Output format: every '>' header line becomes one '\\n' byte; '#' and ';'
start comments that run to the end of the line; spaces, tabs and newlines are
skipped; upper-case letters are copied; anything else is an error naming the
character, its line and the file.  Input may be gzip-compressed.
"""
from __future__ import annotations

import gzip

import numpy as np


class FastaError(RuntimeError):
    pass


_NL, _GT, _HASH, _SEMI, _SP, _TAB = 10, 62, 35, 59, 32, 9


def read_fasta(data: bytes, filename: str = "<bytes>") -> bytes:
    """Returns the residue stream of a FASTA file (ReadFasta.read), vectorised.

    Per line: the first marker ('>', '#', ';') ends the part that is read; a
    '>' marker emits one '\\n' at its position.
    """
    a = np.frombuffer(data, dtype=np.uint8)
    n = len(a)
    if n == 0:
        return b""
    is_nl = a == _NL
    line = np.cumsum(is_nl) - is_nl  # 0-based line of each byte (a newline belongs to its line)
    nlines = int(line[-1]) + 1
    is_mark = (a == _GT) | (a == _HASH) | (a == _SEMI)
    first_mark = np.full(nlines, n, dtype=np.int64)
    mpos = np.flatnonzero(is_mark)
    if len(mpos):
        ml = line[mpos]
        # first marker of each line: positions are ascending, keep the first per line
        first = np.ones(len(mpos), dtype=bool)
        first[1:] = ml[1:] != ml[:-1]
        first_mark[ml[first]] = mpos[first]
    pos = np.arange(n, dtype=np.int64)
    before_mark = pos < first_mark[line]
    keep = before_mark & ~is_nl & (a != _SP) & (a != _TAB)
    header = (pos == first_mark[line]) & (a == _GT)
    bad = keep & ((a < 65) | (a > 90))
    if bad.any():
        i = int(np.argmax(bad))
        raise FastaError(
            f"invalid character '{chr(int(a[i]))}' at line {int(line[i]) + 1} of file '{filename}'")
    out = np.where(header, np.uint8(_NL), a)[keep | header]
    return out.tobytes()


def parse_file_bytes(raw: bytes, filename: str = "<bytes>") -> bytes:
    """parseFiles: gunzip when the data is gzip, then read_fasta."""
    try:
        data = gzip.decompress(raw)
    except (OSError, EOFError, ValueError):
        data = raw
    return read_fasta(data, filename)


def write_fasta(proteins, width: int = 60) -> bytes:
    """Writes proteins (iterable of bytes) as FASTA with '>protein_<i>' headers."""
    parts = []
    for i, p in enumerate(proteins):
        parts.append(b">protein_%d\n" % i)
        for s in range(0, len(p), width):
            parts.append(p[s:s + width] + b"\n")
    return b"".join(parts)

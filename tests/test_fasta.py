"""FASTA ingest semantics of ReadFasta.read (ReadFasta.java:8-46) and
parseFiles (SequenceAnalysisContext.java:60-76)."""
import gzip

import pytest

from rocket_gb300 import fasta


def test_headers_become_newlines():
    src = b">p1 some description\nACDE\nFGH\n>p2\nKLM\n"
    assert fasta.read_fasta(src) == b"\nACDEFGH\nKLM"


def test_comments_whitespace_and_inline_markers():
    src = b"# comment line\n;another\n>h\nAC DE\tF\nGH;trailing comment\nIK#x\n"
    assert fasta.read_fasta(src) == b"\nACDEFGHIK"


def test_header_after_residues_on_same_line():
    assert fasta.read_fasta(b"AC>h\nDE\n") == b"AC\nDE"


def test_invalid_character_reports_line_and_file():
    with pytest.raises(fasta.FastaError) as e:
        fasta.read_fasta(b">h\nACD\nAcD\n", "x.faa")
    assert "invalid character 'c' at line 3 of file 'x.faa'" in str(e.value)
    with pytest.raises(fasta.FastaError):
        fasta.read_fasta(b">h\r\nAC\r\n")  # carriage return is not whitespace here


def test_gzip_and_plain():
    src = b">a\nMKV\n>b\nLLA\n"
    assert fasta.parse_file_bytes(gzip.compress(src)) == b"\nMKV\nLLA"
    assert fasta.parse_file_bytes(src) == b"\nMKV\nLLA"
    assert fasta.read_fasta(b"") == b""


def test_roundtrip_write():
    prots = [b"ACDEFGHIKLMNPQRSTVWY" * 7, b"MKV"]
    assert fasta.read_fasta(fasta.write_fasta(prots)) == b"\n" + prots[0] + b"\n" + prots[1]

"""The distance writer (Main.writeOutput, Main.java:204-251) and the input scan."""
import gzip
import json
import os

import numpy as np

from rocket_gb300.output import scan_directory, write_output


def test_write_output_layout(tmp_path):
    C = np.array([[1.0, 0.25, 0.5], [0.25, 1.0, 0.75], [0.5, 0.75, 1.0]])
    computed = np.ones((3, 3), bool)
    computed[0, 2] = computed[2, 0] = False
    p = tmp_path / "out.json"
    write_output(str(p), ["a.faa", "b.faa", "c.fasta"], C, computed)
    d = json.loads(p.read_text())
    assert d["files"] == ["a.faa", "b.faa", "c.fasta"]
    assert d["distance"][0] == [1.0, 0.25, -1]
    assert d["distance"][2][0] == -1 and d["distance"][1][2] == 0.75


def test_write_output_as_distance(tmp_path):
    C = np.array([[1.0, 0.5], [0.5, 1.0]])
    p = tmp_path / "d.json"
    write_output(str(p), ["x", "y"], C, as_distance=True)
    d = json.loads(p.read_text())
    assert d["distance"] == [[0.0, 0.25], [0.25, 0.0]]


def test_scan_directory_suffixes(tmp_path):
    (tmp_path / "sub").mkdir()
    for name in ("a.faa", "B.FASTA", "sub/c.faa.gz", "d.txt", "e.fasta.gz", "f.fa"):
        path = tmp_path / name
        if name.endswith(".gz"):
            path.write_bytes(gzip.compress(b">x\nAC\n"))
        else:
            path.write_bytes(b">x\nAC\n")
    found = scan_directory(str(tmp_path))
    assert found == sorted(["a.faa", "B.FASTA", os.path.join("sub", "c.faa.gz"), "e.fasta.gz"])

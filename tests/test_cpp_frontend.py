"""The header-only C++20 front-end (include/pairwise_aligner_gb300.hpp).

CPU: it compiles with the reference-style rule nesting and links against the
C ABI library.  GPU: the reference's scalar KATs run through it.
"""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def runner(built_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cpp") / "kat_runner")
    libdir = os.path.dirname(built_lib)
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror",
                           "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "kat_runner.cpp"),
                           "-L", libdir, "-lpa_gb300", f"-Wl,-rpath,{libdir}", "-o", exe])
    return exe


def test_cpp_frontend_compiles_and_links(runner):
    assert os.path.exists(runner)


def _line(c):
    e = lambda k: "1" if c[k] == "free" else "0"
    return " ".join([("1" if c["method"] == "local" else "0"), str(c["gap_open"]), str(c["gap_extension"]),
                     str(c["match"]), str(c["mismatch"]), e("first_column"), e("first_row"), e("last_column"),
                     e("last_row"), c["seq1"] or "-", c["seq2"] or "-"])


def _matrix_line(c, m):
    e = lambda k: "1" if c[k] == "free" else "0"
    scores = " ".join(str(x) for row in m["scores"] for x in row)
    return " ".join(["M", "1" if c["method"] == "local" else "0", str(c["gap_open"]), str(c["gap_extension"]),
                     e("first_column"), e("first_row"), e("last_column"), e("last_row"), str(len(m["symbols"])),
                     "".join(m["symbols"]), scores, c["seq1"] or "-", c["seq2"] or "-"])


@pytest.mark.gpu
def test_cpp_frontend_matrix_kats(runner, matrix_kats):
    """cfg::score_model_matrix with the reference's argument type, BLOSUM62 known answers."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cases = matrix_kats["cases"]
    lines = [_matrix_line(c, matrix_kats["matrices"][c["matrix"]]) for c in cases]
    out = subprocess.run([runner], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout.split("\n")
    for c, line in zip(cases, out):
        assert int(line.split()[0]) == c["expected_score"], (c["source"], c["name"], line)


@pytest.mark.gpu
def test_cpp_frontend_alignments(runner, oracle):
    """compute_alignments through the C++ rule chain equals the oracle's traceback."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pairwise_aligner_gb300 import cigar
    cases = [("ACGTACGT", "ACGTTACGT"), ("ACGT", "AGT"), ("-", "ACG"), ("GATTACA", "GCATGCT"), ("AAAA", "-")]
    lines = [f"T 2 -3 -5 -1 {a} {b}" for a, b in cases]
    out = subprocess.run([runner], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout.split("\n")
    cfg = oracle.make_cfg(2, -3, -5, -1)
    for (a, b), line in zip(cases, out):
        a, b = a.replace("-", ""), b.replace("-", "")
        sc, b1, b2, e1, e2, ops = oracle.traceback(cfg, a.encode(), b.encode())
        assert line.split() == [str(sc), str(b1), str(b2), str(e1), str(e2), cigar(ops) or "-"], (a, b, line)


@pytest.mark.gpu
def test_cpp_frontend_reference_kats(runner, kats):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    out = subprocess.run([runner], input="\n".join(_line(c) for c in kats) + "\n", capture_output=True, text=True,
                         check=True).stdout.split("\n")
    for c, line in zip(kats, out):
        assert int(line.split()[0]) == c["expected_score"], (c["source"], c["name"], line)


def test_cpp_sequence_file_reader(built_lib, tmp_path, oracle):
    """read_sequences / pack_2bit of the C++ front end (host code: runs without a GPU)."""
    import numpy as np
    from pairwise_aligner_gb300 import seqio
    exe = str(tmp_path / "seqfile_dump")
    libdir = os.path.dirname(built_lib)
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror",
                           "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "seqfile_dump.cpp"),
                           "-L", libdir, "-lpa_gb300", f"-Wl,-rpath,{libdir}", "-o", exe])
    text = b"@r1 first\nACGTNACGT\n+\nIIIIIIIII\n@r2\n\n+\n\n@r3\r\nacgtacgtacgtacgtAC\r\n+r3\r\nJJJJJJJJJJJJJJJJJJ\r\n"
    path = tmp_path / "reads.fastq"
    path.write_bytes(text)
    out = subprocess.run([exe, str(path)], capture_output=True, text=True, check=True).stdout.split("\n")
    f = seqio.read_sequences(str(path))
    for k in range(len(f)):
        name, seq, qual = out[k].split("\t")
        q = f.qual[int(f.off[k]):int(f.off[k + 1])].tobytes().decode()
        assert (name, seq, qual) == (f.names[k], f.sequence(k).decode() or "-", q or "-")
    words, bad = oracle.pack_2bit(f.seq)
    assert out[len(f)].split() == [str(int(w)) for w in words] and int(out[len(f) + 1]) == bad
    path.write_bytes(b"@r\nACG\n+\nII\n")
    r = subprocess.run([exe, str(path)], capture_output=True, text=True)
    assert r.returncode == 1 and "line 4" in r.stdout

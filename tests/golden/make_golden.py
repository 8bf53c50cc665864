#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the reference's own tests.

Runs only where the reference checkout is present; the
fixtures it writes are committed, so nothing on a GPU host reads the reference.

* kat_scalar.json -- every unitary-score case of the reference's scalar tests
  (test/unit/affine/*_scalar_test.cpp, test/unit/configuration/*.cpp): the
  configuration, both sequences and the hand-written expected score.
* kat_matrix.json -- the substitution matrices of
  include/pairwise_aligner/score_model/substitution_matrix.hpp (BLOSUM62 over the
  standard and the extended amino-acid alphabets) and every matrix-score case of
  the reference's scalar tests (test/unit/affine/*scalar*test.cpp), with their
  hand-written expected scores.
* simd_differential.json.gz -- every unitary-score case of the reference's SIMD
  tests (test/unit/affine/*_simd_test.cpp).  The reference checks each SIMD
  lane against its scalar aligner on std::mt19937(42) sequences; the sequences
  are regenerated with gen_reference_sequences.cpp (same engine and
  distributions) and the expected scores, plus end coordinates, come from the
  oracle's scalar restatement (oracle/pa_oracle.c), itself pinned by the KATs.
* matrix_differential.json.gz -- the same for the reference's substitution-matrix
  SIMD tests (test/unit/affine/*_simd_matrix_*_test.cpp): BLOSUM62, sequences drawn
  from the matrix's symbol list, one-vs-many cases aligning the first sequence 1
  against every sequence 2.

Usage: python tests/golden/make_golden.py --reference <reference checkout>
(or PA_REFERENCE=<reference checkout> in the environment)
"""
from __future__ import annotations

import argparse
import gzip
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

# AVX-512 lane counts of simd_score<T>::size_v (include/pairwise_aligner/simd/simd_base.hpp:28-36)
LANES = {"int8_t": 64, "int16_t": 32, "int32_t": 16, "int64_t": 8}


def _end_gap(text: str, names: tuple[str, str]) -> dict:
    """Parse leading_end_gap{...} / trailing_end_gap{...} initialisers (end_gap_policy.hpp:26-36)."""
    body = text.strip()
    out = {names[0]: "penalised", names[1]: "penalised"}
    if not body:
        return out
    if "." in body and "=" in body:
        for key, val in re.findall(r"\.(\w+)\s*=\s*[\w:]*end_gap::(\w+)", body):
            out[key] = val
        return out
    vals = re.findall(r"end_gap::(\w+)", body)
    for k, v in zip(names, vals):
        out[k] = v
    return out


def _parse_base_config(src: str, rel: str) -> dict:
    m = re.search(r"base_config\s*=\s*(.*?);\s*\n", src, re.S)
    if not m:
        raise ValueError(f"no base_config in {rel}")
    return _parse_method(m.group(1), rel)


def _call_args(text: str, fn: str):
    """Top-level argument strings of the first call fn(...) in text, or None."""
    k = text.find(fn + "(")
    if k < 0:
        return None
    i, depth, args, cur = k + len(fn) + 1, 1, [], ""
    while depth:
        c = text[i]
        if c in "({":
            depth += 1
        elif c in ")}":
            depth -= 1
        if depth == 1 and c == ",":
            args.append(cur.strip())
            cur = ""
        elif depth:
            cur += c
        i += 1
    args.append(cur.strip())
    return args


def _parse_method(text: str, rel: str) -> dict:
    args = _call_args(text, "gap_model_affine")
    if args is None:
        raise ValueError(f"no gap model in {rel}: {text}")
    cfg = {"gap_open": int(args[-2]), "gap_extension": int(args[-1])}
    if "method_local" in text:
        cfg.update(method="local", first_column="free", first_row="free", last_column="free", last_row="free")
    else:
        lead = re.search(r"leading_end_gap\{(.*?)\}", text, re.S)
        trail = re.search(r"trailing_end_gap\{(.*?)\}", text, re.S)
        cfg["method"] = "global"
        cfg.update(_end_gap(lead.group(1) if lead else "", ("first_column", "first_row")))
        cfg.update(_end_gap(trail.group(1) if trail else "", ("last_column", "last_row")))
    return cfg


def _blocks(src: str):
    """Yield (name, body, line) of each DEFINE_TEST_VALUES(name, ...) macro use."""
    for m in re.finditer(r"DEFINE_TEST_VALUES\((\w+),", src):
        depth, i = 1, m.end()
        while depth:
            c = src[i]
            depth += (c == "(") - (c == ")")
            i += 1
        yield m.group(1), src[m.end():i - 1], src.count("\n", 0, m.start()) + 1


def parse_scalar_kats(ref: str) -> list[dict]:
    cases = []
    d = os.path.join(ref, "test/unit/affine")
    for fn in sorted(os.listdir(d)):
        if not fn.endswith("_scalar_test.cpp") or "matrix" in fn:
            continue
        rel = f"test/unit/affine/{fn}"
        src = open(os.path.join(d, fn)).read()
        base = _parse_base_config(src, rel)
        for name, body, line in _blocks(src):
            conf = re.search(r"\.configurator\s*=\s*(.*?),\s*\n\s*\.sequence1", body, re.S).group(1)
            s1 = re.search(r'\.sequence1\s*=\s*"([^"]*)"sv', body).group(1)
            s2 = re.search(r'\.sequence2\s*=\s*"([^"]*)"sv', body).group(1)
            exp = re.search(r"\.expected_score\s*=\s*([^\n,]+)", body).group(1).strip()
            if "score_model_matrix" in conf:
                if "lowest()" in exp:
                    # empty-sequence rule of the local tracker (tracker_local_scalar.hpp:38); the
                    # rule is independent of the substitution model, so pin it with unitary scores.
                    c = dict(base, match=4, mismatch=-5)
                    cases.append(dict(c, name=name + "_unitary", source=f"{rel}:{line}", seq1=s1, seq2=s2,
                                      expected_score=-2**31))
                continue
            u = re.search(r"score_model_unitary\((.*)\)\s*$", conf.strip(), re.S).group(1)
            scores = re.findall(r"(-?\d+)\s*,\s*(-?\d+)\s*$", u.strip())
            ma, mi = int(scores[0][0]), int(scores[0][1])
            cfg = base if u.strip().startswith("base_config") else _parse_method(u, rel)
            cases.append(dict(cfg, match=ma, mismatch=mi, name=name, source=f"{rel}:{line}", seq1=s1,
                              seq2=s2, expected_score=int(exp)))
    # configuration smoke tests (test/unit/configuration)
    for fn, rel_line in (("configuration_test.cpp", None), ("configure_aligner_saturated_test.cpp", None)):
        rel = f"test/unit/configuration/{fn}"
        src = open(os.path.join(ref, rel)).read()
        body = src[src.index("configure_aligner("):]
        cfg = _parse_method(body, rel)
        sm = re.search(r"score_model_unitary(?:_simd_saturated)?\(\s*(?:\(int16_t\))?(-?\d+)\s*,\s*(?:\(int16_t\))?(-?\d+)", body)
        seqs = re.findall(r'std::string_view seq[12]\{"([^"]*)"\}', src)
        exp = re.search(r"score\(\),\s*(-?\d+)\)", src)
        line = src.count("\n", 0, src.index("configure_aligner(")) + 1
        cases.append(dict(cfg, match=int(sm.group(1)), mismatch=int(sm.group(2)), name=fn[:-4],
                          source=f"{rel}:{line}", seq1=seqs[0], seq2=seqs[1], expected_score=int(exp.group(1))))
    return cases


def parse_substitution_matrices(ref: str) -> dict:
    """{name: {"symbols": [...], "scores": dim x dim}} from substitution_matrix.hpp."""
    src = open(os.path.join(ref, "include/pairwise_aligner/score_model/substitution_matrix.hpp")).read()
    out = {}
    for m in re.finditer(r"(blosum62_\w+)\s*\{\{(.*?)\}\};", src, re.S):
        rows = re.findall(r"\{'(.)',\s*\{([^}]*)\}\}", m.group(2))
        symbols = [r[0] for r in rows]
        scores = [[int(v) for v in r[1].split(",")] for r in rows]
        if any(len(r) != len(symbols) for r in scores):
            raise ValueError(f"{m.group(1)}: matrix is not square")
        out[m.group(1)] = {"symbols": symbols, "scores": scores}
    return out


def parse_matrix_kats(ref: str) -> list[dict]:
    cases = []
    d = os.path.join(ref, "test/unit/affine")
    for fn in sorted(os.listdir(d)):
        if not (fn.endswith("_scalar_test.cpp") or fn.endswith("_scalar_matrix_test.cpp")):
            continue
        rel = f"test/unit/affine/{fn}"
        src = open(os.path.join(d, fn)).read()
        base = _parse_base_config(src, rel)
        for name, body, line in _blocks(src):
            conf = re.search(r"\.configurator\s*=\s*(.*?),\s*\n\s*\.sequence1", body, re.S).group(1)
            mm = re.search(r"score_model_matrix\(\s*base_config\s*,\s*aligner::(blosum62_\w+)<\w*>\s*\)", conf)
            if not mm:
                continue
            s1 = re.search(r'\.sequence1\s*=\s*"([^"]*)"sv', body).group(1)
            s2 = re.search(r'\.sequence2\s*=\s*"([^"]*)"sv', body).group(1)
            exp = re.search(r"\.expected_score\s*=\s*([^\n,]+)", body).group(1).strip()
            expected = -2**31 if "lowest()" in exp else int(exp)
            cases.append(dict(base, matrix=mm.group(1), match=0, mismatch=0, name=name, source=f"{rel}:{line}",
                              seq1=s1, seq2=s2, expected_score=expected))
    return cases


def parse_simd_cases(ref: str) -> list[dict]:
    cases = []
    d = os.path.join(ref, "test/unit/affine")
    for fn in sorted(os.listdir(d)):
        if not fn.endswith("_simd_test.cpp") or "matrix" in fn:
            continue
        rel = f"test/unit/affine/{fn}"
        src = open(os.path.join(d, fn)).read()
        base = _parse_base_config(src, rel)
        count_const = re.search(r"sequence_count\s*=\s*aligner::simd_score<(\w+)>::size_v", src)
        for name, body, line in _blocks(src):
            um = re.search(r"unitary_model<(\w+)>\{(-?\d+),\s*(-?\d+)\}", body)
            if not um:
                continue
            gp = re.search(r"sequence_generation_param\{\s*([^,]+),\s*(\d+),\s*(\d+)\s*\}", body)
            cexpr = gp.group(1).strip()
            if cexpr == "sequence_count":
                count = LANES[count_const.group(1)]
            else:
                count = LANES[re.search(r"simd_score<(\w+)>", cexpr).group(1)]
            kind = "saturated" if "saturated" in body else "fixed"
            cases.append(dict(base, match=int(um.group(2)), mismatch=int(um.group(3)), name=f"{fn[:-9]}:{name}",
                              source=f"{rel}:{line}", score_model=kind, seed=42, count=count,
                              min_size=int(gp.group(2)), max_size=int(gp.group(3))))
    return cases


def parse_matrix_simd_cases(ref: str) -> list[dict]:
    cases = []
    d = os.path.join(ref, "test/unit/affine")
    for fn in sorted(os.listdir(d)):
        if not (fn.endswith("_test.cpp") and "_simd_matrix_" in fn):
            continue
        rel = f"test/unit/affine/{fn}"
        src = open(os.path.join(d, fn)).read()
        base = _parse_base_config(src, rel)
        count_const = re.search(r"sequence_count\s*=\s*aligner::simd_score<(\w+)>::size_v", src)
        for name, body, line in _blocks(src):
            mm = re.search(r"matrix_model\{aligner::(blosum62_\w+)<(\w+)>\}", body)
            if not mm:
                continue
            gp = re.search(r"sequence_generation_param\{\s*([^,]+),\s*(\d+),\s*(\d+)\s*\}", body)
            cexpr = gp.group(1).strip()
            if cexpr == "sequence_count":
                count = LANES[count_const.group(1)]
            else:
                count = LANES[re.search(r"simd_score<(\w+)>", cexpr).group(1)]
            one_vs_many = re.search(r"one_vs_many\s*=\s*std::true_type", body) is not None
            cases.append(dict(base, match=0, mismatch=0, matrix=mm.group(1), score_type=mm.group(2),
                              name=f"{fn[:-9]}:{name}", source=f"{rel}:{line}", seed=42, count=count,
                              min_size=int(gp.group(2)), max_size=int(gp.group(3)), one_vs_many=one_vs_many))
    return cases


def oracle_cfg(c: dict, matrices: dict | None = None):
    from oracle import oracle as O
    mat = None
    if c.get("matrix"):
        m = matrices[c["matrix"]]
        mat = (m["symbols"], m["scores"])
    return O.make_cfg(c["match"], c["mismatch"], c["gap_open"], c["gap_extension"], local=c["method"] == "local",
                      first_column_free=c["first_column"] == "free", first_row_free=c["first_row"] == "free",
                      last_column_free=c["last_column"] == "free", last_row_free=c["last_row"] == "free",
                      matrix=mat)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("PA_REFERENCE"),
                    help="the reference checkout (default: $PA_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference or set PA_REFERENCE")
    from oracle import oracle as O

    kats = parse_scalar_kats(args.reference)
    for k in kats:                       # the oracle must reproduce every hand-written score
        sc, _, _ = O.align(oracle_cfg(k), k["seq1"].encode(), k["seq2"].encode())
        if sc != k["expected_score"]:
            raise SystemExit(f"oracle disagrees with {k['source']} {k['name']}: {sc} != {k['expected_score']}")
    with open(os.path.join(HERE, "kat_scalar.json"), "w") as f:
        json.dump(kats, f, indent=1)
    print(f"kat_scalar.json: {len(kats)} cases, oracle agrees with all")

    matrices = parse_substitution_matrices(args.reference)
    mkats = parse_matrix_kats(args.reference)
    for k in mkats:
        if not k["seq1"] or not k["seq2"]:
            if k["method"] == "local" and k["expected_score"] == -2**31:
                continue                 # the empty-sequence rule; the oracle returns it for any model
        sc, _, _ = O.align(oracle_cfg(k, matrices), k["seq1"].encode(), k["seq2"].encode())
        if sc != k["expected_score"]:
            raise SystemExit(f"oracle disagrees with {k['source']} {k['name']}: {sc} != {k['expected_score']}")
    with open(os.path.join(HERE, "kat_matrix.json"), "w") as f:
        json.dump({"matrices": matrices, "cases": mkats}, f, indent=1)
    print(f"kat_matrix.json: {len(matrices)} matrices, {len(mkats)} cases, oracle agrees with all")

    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "gen")
        subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(HERE, "gen_reference_sequences.cpp"),
                               "-o", exe])
        cases = parse_simd_cases(args.reference)
        for c in cases:
            out = subprocess.check_output([exe, str(c["seed"]), str(c["count"]), str(c["min_size"]),
                                           str(c["max_size"])]).decode().split("\n")
            s1, s2 = out[:c["count"]], out[c["count"]:2 * c["count"]]
            c["seqs1"], c["seqs2"] = s1, s2
            res = [O.align(oracle_cfg(c), a.encode(), b.encode()) for a, b in zip(s1, s2)]
            c["oracle_scores"] = [r[0] for r in res]
            c["oracle_end1"] = [r[1] for r in res]
            c["oracle_end2"] = [r[2] for r in res]
        mcases = parse_matrix_simd_cases(args.reference)
        for c in mcases:
            symbols = "".join(matrices[c["matrix"]]["symbols"])
            out = subprocess.check_output([exe, str(c["seed"]), str(c["count"]), str(c["min_size"]),
                                           str(c["max_size"]), symbols]).decode().split("\n")
            s1, s2 = out[:c["count"]], out[c["count"]:2 * c["count"]]
            if c["one_vs_many"]:
                s1 = [s1[0]] * len(s2)          # sequence1() is the first of collection 1
            c["seqs1"], c["seqs2"] = s1, s2
            res = [O.align(oracle_cfg(c, matrices), a.encode(), b.encode()) for a, b in zip(s1, s2)]
            c["oracle_scores"] = [r[0] for r in res]
            c["oracle_end1"] = [r[1] for r in res]
            c["oracle_end2"] = [r[2] for r in res]
    with gzip.open(os.path.join(HERE, "simd_differential.json.gz"), "wt") as f:
        json.dump(cases, f)
    print(f"simd_differential.json.gz: {len(cases)} cases, {sum(c['count'] for c in cases)} pairs")
    with gzip.open(os.path.join(HERE, "matrix_differential.json.gz"), "wt") as f:
        json.dump(mcases, f)
    print(f"matrix_differential.json.gz: {len(mcases)} cases, {sum(c['count'] for c in mcases)} pairs")
    return 0


if __name__ == "__main__":
    sys.exit(main())

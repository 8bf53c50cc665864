"""The input path: FASTA / FASTQ reader, rank map, 2-bit packing, packed alignment.

CPU: the native reader against a Python restatement of the record format on random
files (CRLF, empty records, wrapped FASTA), its error reports, and the host 2-bit
encoder against the oracle's numpy restatement.  GPU: the rank-map kernel on the
reference's symbol lists (alphabet_rank_map_simd_test.cpp: smallest / largest rank,
ranks in order and reversed) and on random bytes, the pack / unpack kernels at any
alignment, and pa_align_batch_packed against pa_align_batch.
"""
from __future__ import annotations

import numpy as np
import pytest

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


# -- a Python restatement of the record format ----------------------------------------------------

def _py_parse(text: bytes):
    lines = [ln.rstrip(b"\r \t") for ln in text.split(b"\n")]
    i = 0
    while i < len(lines) and not lines[i]:
        i += 1
    if i == len(lines):
        return [], [], None
    names, seqs, quals = [], [], []
    if lines[i][:1] == b">":
        cur = None
        for ln in lines[i:]:
            if ln[:1] == b">":
                if cur is not None:
                    seqs.append(b"".join(cur))
                names.append(ln[1:].decode())
                cur = []
            elif ln:
                cur.append(ln.replace(b" ", b"").replace(b"\t", b""))
        seqs.append(b"".join(cur))
        return names, seqs, None
    while i < len(lines):
        if not lines[i]:
            i += 1
            continue
        names.append(lines[i][1:].decode())
        i += 1
        s = []
        while not lines[i][:1] == b"+":
            s.append(lines[i])
            i += 1
        i += 1
        seq = b"".join(s)
        q = []
        while sum(map(len, q)) < len(seq):
            q.append(lines[i])
            i += 1
        seqs.append(seq)
        quals.append(b"".join(q))
    return names, seqs, quals


def _random_text(rng, fastq: bool, crlf: bool, n_records: int = 40):
    eol = b"\r\n" if crlf else b"\n"
    out = []
    for k in range(n_records):
        n = int(rng.integers(0, 300)) if k % 7 else 0
        seq = ACGT[rng.integers(0, 4, n)].tobytes()
        name = f"read_{k} len={n}".encode()
        if fastq:
            qual = rng.integers(33, 74, n).astype(np.uint8).tobytes()
            out += [b"@" + name, seq, b"+" + (name if k % 2 else b""), qual]
        else:
            width = int(rng.integers(1, 80))
            out.append(b">" + name)
            out += [seq[i:i + width] for i in range(0, len(seq), width)] or [b""]
    return eol.join(out) + eol


@pytest.mark.parametrize("fastq", [True, False])
@pytest.mark.parametrize("crlf", [False, True])
def test_reader_matches_restatement(built_lib, fastq, crlf):
    from pairwise_aligner_gb300 import seqio
    rng = np.random.default_rng(1 + 2 * fastq + crlf)
    text = _random_text(rng, fastq, crlf)
    f = seqio.parse_sequences(text)
    names, seqs, quals = _py_parse(text)
    assert f.names == names
    assert [f.sequence(i) for i in range(len(f))] == seqs
    if fastq:
        assert [f.qual[int(f.off[i]):int(f.off[i + 1])].tobytes() for i in range(len(f))] == quals
    else:
        assert f.qual is None


def test_reader_file_and_empty_input(built_lib, tmp_path):
    from pairwise_aligner_gb300 import seqio
    text = _random_text(np.random.default_rng(5), True, False, 10)
    p = tmp_path / "reads.fastq"
    p.write_bytes(text)
    a, b = seqio.read_sequences(str(p)), seqio.parse_sequences(text)
    assert a.names == b.names and np.array_equal(a.seq, b.seq) and np.array_equal(a.off, b.off)
    for empty in (b"", b"\n\n  \n"):
        f = seqio.parse_sequences(empty)
        assert len(f) == 0 and list(f.off) == [0]


@pytest.mark.parametrize("text,line", [(b"ACGT\n", 1), (b"@r\nACG\n+\nII\n", 4), (b"@r\nACG\nIII\n", 3),
                                       (b"@r\nACG\n+\nIIII\n", 4), (b"@a\nAC\n+\nII\nxx\n", 5),
                                       (b"\n\n#comment\n", 3)])
def test_reader_reports_malformed_records(built_lib, text, line):
    from pairwise_aligner_gb300 import PaError, seqio
    with pytest.raises(PaError) as e:
        seqio.parse_sequences(text)
    assert e.value.status == 1 and f"line {line}:" in str(e.value)


def test_reader_missing_file(built_lib, tmp_path):
    from pairwise_aligner_gb300 import PaError, seqio
    with pytest.raises(PaError):
        seqio.read_sequences(str(tmp_path / "absent.fa"))


def test_host_packer_matches_oracle(built_lib, oracle):
    from pairwise_aligner_gb300 import seqio
    rng = np.random.default_rng(6)
    letters = np.frombuffer(b"ACGTacgt", dtype=np.uint8)
    for n in [0, 1, 15, 16, 17, 31, 33, 1000, 65537]:
        x = rng.integers(0, 256, n).astype(np.uint8)
        m = rng.random(n) < 0.8
        x[m] = letters[rng.integers(0, 8, int(m.sum()))]
        w, bad = seqio.pack_2bit(x)
        ow, obad = oracle.pack_2bit(x)
        assert np.array_equal(w, ow) and bad == obad, n


def test_oracle_rank_table_follows_reference_rules(oracle):
    t = oracle.rank_table(b"ACGTN")
    assert [t[c] for c in b"ACGTN"] == [0, 1, 2, 3, 4] and t[ord("a")] == -1
    assert oracle.rank_table(b"ABA")[ord("A")] == 2               # the last rank of a repeat
    with pytest.raises(ValueError):
        oracle.rank_table(b"")


# -- GPU ------------------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def pa(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pairwise_aligner_gb300 as pa
    return pa


SYMBOL_LISTS = [b"X", b"ACGTN", b"ACDEFGHIKLMNPQRSTVWY", b"ABCDEFGHIJKLMNOPQRSTUVWXYZ*",
                bytes(range(32, 127))]      # the printable characters


@pytest.mark.gpu
@pytest.mark.parametrize("symbols", SYMBOL_LISTS)
def test_rank_map_reference_rules(pa, oracle, symbols):
    """smallest_rank / largest_rank / rank_in_order / rank_in_reversed_order of the reference's
    alphabet_rank_map_simd_test.cpp, on 64-symbol keys as its int8 SIMD vectors hold."""
    import torch
    ctx = pa.Context(0)
    keys = []
    keys.append(bytes([symbols[0]]) * 64)
    keys.append(bytes([symbols[-1]]) * 64)
    for j in range(0, len(symbols), 64):
        sl = symbols[j:j + 64]
        keys.append(bytes(sl[i % len(sl)] for i in range(64)))
        keys.append(bytes(sl[i % len(sl)] for i in range(64))[::-1])
    data = np.frombuffer(b"".join(keys), dtype=np.uint8)
    d_in = torch.from_numpy(data.copy()).cuda()
    d_out = torch.empty(len(data), dtype=torch.int8, device="cuda")
    bad = pa.seqio.rank_map_device(ctx, symbols, d_in, d_out, count_invalid=True)
    got = d_out.cpu().numpy()
    assert bad == 0
    assert np.array_equal(got, oracle.rank_map(symbols, data))
    assert (got[:64] == 0).all() and (got[64:128] == len(symbols) - 1).all()


@pytest.mark.gpu
def test_rank_map_random_bytes_any_alignment(pa, oracle):
    import torch
    rng = np.random.default_rng(7)
    ctx = pa.Context(0)
    symbols = b"ACDEFGHIKLMNPQRSTVWY"
    big = rng.integers(0, 256, 3 * (1 << 20) + 77).astype(np.uint8)
    d_big = torch.from_numpy(big).cuda()
    d_out = torch.empty(len(big) + 64, dtype=torch.int8, device="cuda")
    for start, n, ostart in [(0, len(big), 0), (1, 1000, 0), (3, 4096, 5), (0, 15, 0), (16, 17, 16), (0, 0, 0),
                             (9, len(big) - 9, 7)]:
        bad = pa.seqio.rank_map_device(ctx, symbols, d_big[start:start + n], d_out[ostart:ostart + n],
                                       count_invalid=True)
        want = oracle.rank_map(symbols, big[start:start + n])
        assert np.array_equal(d_out[ostart:ostart + n].cpu().numpy(), want), (start, n, ostart)
        assert bad == int((want < 0).sum())
    with pytest.raises(pa.PaError):
        pa.seqio.rank_map_device(ctx, b"", d_big[:10], d_out[:10])


@pytest.mark.gpu
def test_pack_and_unpack_kernels(pa, oracle):
    import torch
    rng = np.random.default_rng(8)
    ctx = pa.Context(0)
    letters = np.frombuffer(b"ACGTacgtN", dtype=np.uint8)
    x = letters[rng.integers(0, 9, 5 * (1 << 20) + 13)]
    d_x = torch.from_numpy(x).cuda()
    d_w = torch.zeros(len(x) // 16 + 2, dtype=torch.int32, device="cuda")
    for start, n in [(0, len(x)), (1, 999), (7, 16), (0, 1), (5, 0), (16, 4097)]:
        d_w.zero_()
        bad = pa.seqio.pack_2bit_device(ctx, d_x[start:start + n], d_w, count_invalid=True)
        ow, obad = oracle.pack_2bit(x[start:start + n])
        got = d_w[:len(ow)].cpu().numpy().view(np.uint32)
        assert np.array_equal(got, ow) and bad == obad, (start, n)
    # unpack: any first base, any length; letters come back upper-case
    clean = ACGT[rng.integers(0, 4, 200_003)]
    words, _ = oracle.pack_2bit(clean)
    d_words = torch.from_numpy(words.view(np.int32).copy()).cuda()
    d_out = torch.zeros(len(clean) + 32, dtype=torch.uint8, device="cuda")
    for first, n, ostart in [(0, len(clean), 0), (1, 100, 0), (15, 1000, 3), (16, 33, 16), (37, 0, 0),
                             (5, len(clean) - 5, 1)]:
        pa.seqio.unpack_2bit_device(ctx, d_words, first, n, d_out[ostart:])
        torch.cuda.synchronize()
        assert np.array_equal(d_out[ostart:ostart + n].cpu().numpy(), clean[first:first + n]), (first, n)


@pytest.mark.gpu
@pytest.mark.parametrize("local", [False, True])
def test_packed_alignment_equals_byte_alignment(pa, local):
    from pairwise_aligner_gb300 import pack, seqio
    rng = np.random.default_rng(9 + local)
    shapes = [(int(rng.integers(0, 600)), int(rng.integers(0, 600))) for _ in range(3000)]
    shapes += [(2500, 2600), (17, 4000), (0, 0)]
    s1 = [ACGT[rng.integers(0, 4, m)].tobytes() for m, _ in shapes]
    s2 = [ACGT[rng.integers(0, 4, n)].tobytes() for _, n in shapes]
    q, qo = pack(s1)
    t, to = pack(s2)
    c = dict(local=local, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, first_column_free=local,
             first_row_free=local, last_column_free=local, last_row_free=local)
    al = pa.Aligner(c)
    want = al.compute_arrays(q, qo, t, to).copy()
    w1, _ = seqio.pack_2bit(q)
    w2, _ = seqio.pack_2bit(t)
    got = al.compute_packed(w1, qo, w2, to)
    for f in ("score", "end1", "end2"):
        assert np.array_equal(got[f], want[f])
    # a slice of the batch: offsets that start inside a packed word
    k0, k1 = 101, 2000
    got = al.compute_packed(w1, qo[k0:k1 + 1], w2, to[k0:k1 + 1])
    for f in ("score", "end1", "end2"):
        assert np.array_equal(got[f], want[f][k0:k1])


@pytest.mark.gpu
def test_fastq_records_aligned_against_oracle(pa, oracle, tmp_path):
    from pairwise_aligner_gb300 import seqio
    rng = np.random.default_rng(11)
    text = _random_text(rng, True, False, 200)
    p = tmp_path / "r.fastq"
    p.write_bytes(text)
    f = seqio.read_sequences(str(p))
    n = len(f) // 2
    # pair k: record 2k against record 2k+1
    s1 = np.concatenate([f.seq[int(f.off[2 * k]):int(f.off[2 * k + 1])] for k in range(n)])
    o1 = np.concatenate([[0], np.cumsum([int(f.off[2 * k + 1] - f.off[2 * k]) for k in range(n)])]).astype(np.uint64)
    s2 = np.concatenate([f.seq[int(f.off[2 * k + 1]):int(f.off[2 * k + 2])] for k in range(n)])
    o2 = np.concatenate([[0], np.cumsum([int(f.off[2 * k + 2] - f.off[2 * k + 1]) for k in range(n)])]).astype(np.uint64)
    res = pa.Aligner(dict(local=True, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, first_column_free=True,
                          first_row_free=True, last_column_free=True, last_row_free=True)).compute_arrays(s1, o1, s2, o2)
    sc, e1, e2 = oracle.align_batch(oracle.make_cfg(2, -3, -5, -1, local=True), s1, o1, s2, o2)
    assert np.array_equal(res["score"], sc) and np.array_equal(res["end1"], e1) and np.array_equal(res["end2"], e2)

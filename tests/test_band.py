"""The learned band: labels, features and the MLP's forward/backward kernels.

CPU tests pin the label definition of the oracle; GPU tests compare the
labeller (full GPU DP in its label modes) with the oracle, the 12-mer diagonal
histogram kernel with a numpy restatement, and the BF16 MLP kernels with a numpy
model of the same network that rounds to BF16 where the kernels do.
"""
import numpy as np
import pytest

from pairwise_aligner_gb300 import workloads

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def _aligner(d):
    from pairwise_aligner_gb300 import Aligner
    return Aligner(dict(local=d["local"], match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                        gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                        last_column_free=False, last_row_free=False))


def _pair(d, k):
    a = bytes(d["seq1"][d["off1"][k]:d["off1"][k + 1]])
    b = bytes(d["seq2"][d["off2"][k]:d["off2"][k + 1]])
    return a, b


# ---------------------------------------------------------------------------- CPU
def test_oracle_labels_identity_and_shift(oracle):
    cfg = oracle.make_cfg(1, -4, -6, -1)
    rng = np.random.default_rng(7)
    s = bytes(ACGT[rng.integers(0, 4, 300)])
    assert oracle.band_labels(cfg, s, s) == [0] * 8
    ins = bytes(ACGT[rng.integers(0, 4, 60)])
    lab = oracle.band_labels(cfg, s, ins + s)           # sequence2 starts with 60 extra bases
    assert lab == [60] * 8
    assert oracle.band_labels(cfg, s[:8], s) == [0] * 8     # too short: no checkpoints


def test_targets_and_centres_round_trip():
    from pairwise_aligner_gb300 import band
    lab = np.array([[0, 3, -5, 40, 40, 41, 39, 38]], dtype=np.int32)
    m, n = np.array([300]), np.array([338])
    y = band.targets(lab, m, n, score=np.array([100]), smax=1)
    d, c2 = band.band_centres(y, m, n)
    assert (d == lab).all()
    assert abs(c2[0] - (638 - 200)) < 1e-6 * 638


def _bf16(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def _features_np(a: bytes, b: bytes) -> np.ndarray:
    """Numpy restatement of k_kmer_hist (no subsampling: len(b) <= 6000)."""
    m, n = len(a), len(b)
    code = {65: 0, 67: 1, 71: 2, 84: 3}
    first = {}
    for j in range(0, n - 11):
        w = b[j:j + 12]
        if all(c in code for c in w):
            first.setdefault(w, j)
    hist = np.zeros(128, np.uint32)
    nq = 0
    for i in range(0, m - 11):
        w = a[i:i + 12]
        if not all(c in code for c in w):
            continue
        nq += 1
        if w in first:
            bin_ = ((first[w] - i + m) * 128) // (m + n + 1)
            hist[min(max(bin_, 0), 127)] += 1
    f = np.zeros(130, np.float32)
    norm = np.float32(1.0) / np.float32(max(nq, 1))
    f[:128] = hist.astype(np.float32) * norm
    f[128] = np.float32(m) / np.float32(1024)
    f[129] = np.float32(n) / np.float32(1024)
    return f


def _mlp_np(st, x, y, mask):
    """Forward + backward of the band MLP in numpy with the kernels' BF16 rounding points."""
    B = x.shape[0]
    x16 = np.zeros((B, 144), np.float32)
    x16[:, :130] = _bf16(x)
    W1, W2, W3 = _bf16(st["W1"]), _bf16(st["W2"]), _bf16(st["W3"])
    h1 = _bf16(np.maximum(x16 @ W1 + st["b1"], 0))
    h2 = _bf16(np.maximum(h1 @ W2 + st["b2"], 0))
    out = h2 @ W3 + st["b3"]
    scale = np.float32(2.0) / (np.float32(B) * np.float32(9))
    d = np.zeros((B, 16), np.float32)
    d[:, :9] = (out[:, :9] - y) * (mask[:, None] != 0)
    dout = _bf16(d * scale)
    g = {"W3": h2.T @ dout, "b3": dout.sum(0)}
    dh2 = _bf16(dout @ W3.T) * (h2 > 0)
    g["W2"], g["b2"] = h1.T @ dh2, dh2.sum(0)
    dh1 = _bf16(dh2 @ W2.T) * (h1 > 0)
    g["W1"], g["b1"] = x16.T @ dh1, dh1.sum(0)
    return out, g, float((d[:, :9] ** 2).sum())


# ---------------------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_gpu_labels_match_oracle(oracle):
    from pairwise_aligner_gb300 import band
    d = workloads.subset(workloads.config4(seed=41, n_pairs=512), np.arange(48))
    al = _aligner(d)
    lab = band.labels(al.context, al.c_config(), d["seq1"], d["off1"], d["seq2"], d["off2"])
    cfg = oracle.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"])
    for k in range(len(d["off1"]) - 1):
        a, b = _pair(d, k)
        assert list(lab[k]) == oracle.band_labels(cfg, a, b), k


@pytest.mark.gpu
def test_gpu_labels_edge_shapes(oracle):
    from pairwise_aligner_gb300 import band
    rng = np.random.default_rng(3)
    lens = [(9, 1), (8, 50), (0, 5), (5, 0), (40, 300), (300, 40), (1000, 1100), (9, 9)]
    s1 = [bytes(ACGT[rng.integers(0, 4, a)]) for a, _ in lens]
    s2 = [bytes(ACGT[rng.integers(0, 4, b)]) for _, b in lens]
    off1 = np.concatenate([[0], np.cumsum([len(x) for x in s1])]).astype(np.uint64)
    off2 = np.concatenate([[0], np.cumsum([len(x) for x in s2])]).astype(np.uint64)
    al = _aligner(dict(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1))
    lab = band.labels(al.context, al.c_config(), np.frombuffer(b"".join(s1), np.uint8), off1,
                      np.frombuffer(b"".join(s2), np.uint8), off2)
    cfg = oracle.make_cfg(2, -3, -5, -1)
    for k in range(len(lens)):
        assert list(lab[k]) == oracle.band_labels(cfg, s1[k], s2[k]), lens[k]


@pytest.mark.gpu
def test_gpu_features_match_numpy():
    import torch
    from pairwise_aligner_gb300 import band
    d = workloads.subset(workloads.config4(seed=42, n_pairs=256), np.arange(40))
    # a few non-ACGT bytes so the k-mer validity rule is exercised
    d["seq1"] = d["seq1"].copy()
    d["seq1"][5::97] = ord("N")
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(d[k])).to(dev) for k in ("seq1", "seq2")}
    o = {k: torch.from_numpy(d[k].astype(np.int64)).to(dev) for k in ("off1", "off2")}
    f = band.features(t["seq1"], o["off1"], t["seq2"], o["off2"]).cpu().numpy()
    for k in range(40):
        a, b = _pair(d, k)
        np.testing.assert_array_equal(f[k], _features_np(a, b), err_msg=str(k))


@pytest.mark.gpu
def test_gpu_mlp_forward_backward_against_numpy():
    import torch
    from pairwise_aligner_gb300 import band
    rng = np.random.default_rng(5)
    B = 96                                           # not a multiple of the 64-row tile
    model = band.BandModel(seed=11, max_batch=B)
    st = model.state()
    for k in ("b1", "b2"):
        st[k] = rng.standard_normal(st[k].shape).astype(np.float32) * 0.1
    st["b3"][:9] = rng.standard_normal(9).astype(np.float32) * 0.1
    model.load_state(st)
    x = rng.random((B, 130), dtype=np.float32)
    y = rng.standard_normal((B, 9)).astype(np.float32)
    mask = (rng.random(B) > 0.1).astype(np.float32)
    dev = model.dev
    out = model.forward(torch.from_numpy(x).to(dev), B).cpu().numpy()
    model.backward(torch.from_numpy(y).to(dev), torch.from_numpy(mask).to(dev), B)
    torch.cuda.synchronize()
    ref_out, ref_g, ref_loss = _mlp_np(st, x, y, mask)
    np.testing.assert_allclose(out[:, :9], ref_out[:, :9], rtol=2e-2, atol=2e-2)
    assert abs(float(model.loss.item()) - ref_loss) <= 2e-2 * max(1.0, ref_loss)
    for k, g in ref_g.items():
        got = model.g[k].cpu().numpy()
        scale = float(np.abs(g).max()) + 1e-12
        # BF16 activations: one rounding step may differ where fp32 sums are ordered differently
        assert np.abs(got - g).max() <= 3e-2 * scale, k


@pytest.mark.gpu
def test_gpu_mlp_training_reduces_loss():
    import torch
    from pairwise_aligner_gb300 import band
    rng = np.random.default_rng(9)
    n = 8192
    x = rng.random((n, 130), dtype=np.float32)
    w = rng.standard_normal((130, 9)).astype(np.float32) * 0.3
    y = np.tanh(x @ w).astype(np.float32)
    model = band.BandModel(seed=1, max_batch=1024)
    hist = model.train(x, y, np.ones(n, np.float32), epochs=8, batch=1024, lr=2e-3)
    assert hist[-1] < 0.25 * hist[0], hist
    p = model.predict(torch.from_numpy(x[:100]).to(model.dev))
    assert np.abs(p - y[:100]).mean() < 0.2


# ---------------------------------------------------------------------------- band mode
BANDED, FULL, TRIVIAL = 0x02, 0x04, 0x08


def _check_exact(oracle, d, res):
    cfg = oracle.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"])
    sc, e1, e2 = oracle.align_batch(cfg, d["seq1"], d["off1"], d["seq2"], d["off2"])
    bad = np.flatnonzero((res["score"] != sc) | (res["end1"] != e1) | (res["end2"] != e2))
    assert len(bad) == 0, (len(bad), bad[:5], res[bad[:5]], sc[bad[:5]])
    kinds = (res["flags"] & (BANDED | FULL | TRIVIAL))
    assert np.isin(kinds, [BANDED, FULL, TRIVIAL]).all()       # exactly one outcome per pair


def _low_divergence(seed, n_pairs, lo, hi, div):
    rng = np.random.default_rng(seed)
    m = rng.integers(lo, hi + 1, size=n_pairs)
    q, qo = workloads.random_codes(rng, m)
    t, to = workloads.mutate(rng, q, qo, div * 0.8, div * 0.1, div * 0.1, 2.0)
    return workloads._finish(q, qo, t, to, 5, "low_divergence")


def _true_bands(oracle, d, al, margin=1.5, w_min=16):
    """Bands from the optimal path (labels) and the true score deficit."""
    from pairwise_aligner_gb300 import band
    lab = band.labels(al.context, al.c_config(), d["seq1"], d["off1"], d["seq2"], d["off2"])
    sc = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])["score"].astype(np.int64)
    m = np.diff(d["off1"].astype(np.int64))
    n = np.diff(d["off2"].astype(np.int64))
    smax = max(d["match"], 0)
    c2 = smax * (m + n) - 2 * sc
    per = -d["gap_extension"] + smax
    ws = np.maximum((c2 / 2 + 2 * d["gap_open"]) / per, 0) * margin + w_min
    b = np.zeros((len(m), 10), np.int32)
    b[:, :8] = lab
    b[:, 8] = np.minimum(ws, np.maximum(m, n) + 1).astype(np.int32)
    b[:, 9] = w_min
    return b


@pytest.mark.gpu
def test_gpu_band_certifies_low_divergence_exactly(oracle):
    d = _low_divergence(31, 600, 1500, 4000, 0.02)
    al = _aligner(d)
    bands = _true_bands(oracle, d, al)
    res = al.compute_banded(d["seq1"], d["off1"], d["seq2"], d["off2"], bands)
    _check_exact(oracle, d, res)
    st = al.last_stats
    assert st["pairs_banded"] > 0.8 * 600, st
    assert st["pairs_banded"] + st["pairs_full_dp"] + st["pairs_trivial"] == 600
    assert 0 < st["band_cells"] < 0.6 * st["cells"], st


@pytest.mark.gpu
def test_gpu_band_wrong_bands_stay_exact(oracle):
    """Bands that miss the optimal path or are far too narrow: the certificate must refuse them
    (then doubling or the full DP answers), never accept a wrong score."""
    rng = np.random.default_rng(8)
    d = workloads.subset(workloads.config4(seed=44, n_pairs=2048), np.arange(400))
    d2 = _low_divergence(32, 200, 800, 3000, 0.03)
    al = _aligner(d)
    for dd in (d, d2):
        n = len(dd["off1"]) - 1
        b = np.zeros((n, 10), np.int32)
        b[:, :8] = rng.integers(-300, 300, size=(n, 8))
        b[:, 8] = rng.integers(1, 40, size=n)
        b[:, 9] = 1
        res = al.compute_banded(dd["seq1"], dd["off1"], dd["seq2"], dd["off2"], b)
        _check_exact(oracle, dd, res)
    for w0 in (1, 4):                 # straight centre, tiny widths, every round count
        for rounds in (0, 1, 3, 8):
            al.context.set_band_options(max_rounds=rounds, w_min=1, full_frac=0.9)
            b = np.zeros((len(d2["off1"]) - 1, 10), np.int32)
            b[:, 8], b[:, 9] = w0, 1
            res = al.compute_banded(d2["seq1"], d2["off1"], d2["seq2"], d2["off2"], b)
            _check_exact(oracle, d2, res)
            if rounds == 0:
                assert (res["flags"] & FULL).all()


@pytest.mark.gpu
def test_gpu_band_straight_mode_mixed_stream(oracle):
    d = workloads.config5(seed=55, n_pairs=300, strata=(0.80, 0.15, 0.05))
    cfgd = dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                last_column_free=False, last_row_free=False, band_mode=2)
    from pairwise_aligner_gb300 import Aligner
    al = Aligner(cfgd)
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check_exact(oracle, d, res)
    st = al.last_stats
    assert st["pairs_banded"] + st["pairs_full_dp"] + st["pairs_trivial"] == 300


@pytest.mark.gpu
def test_gpu_band_edge_cases(oracle):
    """Empty, tiny and lopsided pairs, non-ACGT bytes, forced s32 lanes."""
    rng = np.random.default_rng(12)
    shapes = [(0, 0), (0, 7), (7, 0), (1, 1), (3, 50), (50, 3), (8, 9), (9, 8), (200, 1200), (1200, 200),
              (129, 129), (128, 129), (5000, 5100), (4000, 3000)]
    s1, s2 = [], []
    for a, b in shapes:
        x = bytes(ACGT[rng.integers(0, 4, a)])
        y = bytearray(x[: min(a, b)] + bytes(ACGT[rng.integers(0, 4, max(0, b - a))]))
        s1.append(x)
        s2.append(bytes(y[:b]))
    s2[-1] = s2[-1][:100] + b"N" + s2[-1][101:]           # byte-compare class
    from pairwise_aligner_gb300 import Aligner, pack
    q, qo = pack(s1)
    t, to = pack(s2)
    d = dict(seq1=q, off1=qo, seq2=t, off2=to, match=2, mismatch=-3, gap_open=-5, gap_extension=-1)
    for hint in (0, 32):
        al = Aligner(dict(local=False, match=2, mismatch=-3, gap_open=-5, gap_extension=-1, first_column_free=False,
                          first_row_free=False, last_column_free=False, last_row_free=False, width_hint=hint,
                          band_mode=2))
        al.context.set_band_options(straight_w0=8, w_min=2)
        res = al.compute_arrays(q, qo, t, to)
        _check_exact(oracle, d, res)


@pytest.mark.gpu
def test_gpu_band_learned_mode_is_exact_with_any_model(oracle):
    from pairwise_aligner_gb300 import Aligner, PaError, band
    d = workloads.subset(workloads.config4(seed=45, n_pairs=1024), np.arange(300))
    cfgd = dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                last_column_free=False, last_row_free=False, band_mode=1)
    al = Aligner(cfgd)
    with pytest.raises(PaError):              # no model loaded
        al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    band.BandModel(seed=3, max_batch=256).to_context(al.context)      # untrained weights
    res = al.compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
    _check_exact(oracle, d, res)


@pytest.mark.gpu
def test_gpu_band_mode_rejects_local_and_free_ends():
    from pairwise_aligner_gb300 import Aligner, PaError
    base = dict(local=False, match=1, mismatch=-4, gap_open=-6, gap_extension=-1, first_column_free=False,
                first_row_free=False, last_column_free=False, last_row_free=False, band_mode=2)
    for change in (dict(local=True), dict(last_row_free=True), dict(first_column_free=True)):
        al = Aligner({**base, **change})
        with pytest.raises(PaError):
            al.compute([b"ACGTACGT"], [b"ACGTTCGT"])


@pytest.mark.gpu
def test_gpu_learned_band_gains_over_straight_band():
    """What the network gains: on a fixed mixed-stream sample with 128-ish very long pairs
    (20-50 kb, 6 % divergence, one or two 50-500 bp structural indels each), the trained
    predictor's bands certify most very long pairs within one doubling.  Straight bands along
    the main diagonal (band_mode 2, the same certificate and doubling) certify none of them
    before they pass full_frac of the matrix.  Both modes return the plain path's results."""
    import os
    import torch
    import pairwise_aligner_gb300 as pa
    from pairwise_aligner_gb300 import Aligner, band
    d = workloads.config5(seed=77, n_pairs=256, strata=(0.2, 0.3, 0.5))
    very_long = d["stratum"] == 2
    assert very_long.sum() >= 100
    base = dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                last_column_free=False, last_row_free=False, band_mode=0)
    args = (d["seq1"], d["off1"], d["seq2"], d["off2"])
    plain = Aligner(base).compute_arrays(*args)
    got = {}
    for mode in (1, 2):
        al = Aligner({**base, "band_mode": mode})
        if mode == 1:
            model = band.BandModel(device=torch.device("cuda:0"))
            model.load(os.path.join(os.path.dirname(pa.__file__), "data", "band_model.npz"))
            model.to_context(al.context)
        res = al.compute_arrays(*args)
        for f in ("score", "end1", "end2"):
            assert np.array_equal(res[f], plain[f]), (mode, f)
        got[mode] = res
    cert = {k: ((r["flags"] & BANDED) != 0) & very_long for k, r in got.items()}
    n_long = int(very_long.sum())
    assert cert[1].sum() >= 0.6 * n_long, (int(cert[1].sum()), n_long)
    assert cert[2].sum() <= 0.1 * n_long, (int(cert[2].sum()), n_long)
    assert got[1]["band_rounds"][cert[1]].mean() <= 1.0        # round 0 or one doubling


@pytest.mark.gpu
def test_gpu_band_mode_device_entry_without_stats():
    """Band mode through pa_align_batch_device without a stats block returns once its last
    launches are queued; after a stream sync the results equal the plain path's, for a batch
    with long pairs (band rounds, concurrent long and largest classes, full-DP leftovers) and
    for one without (short pairs only), twice in a row on the same buffers."""
    import os
    import torch
    import pairwise_aligner_gb300 as pa
    from pairwise_aligner_gb300 import Aligner, band
    dev = torch.device("cuda:0")
    model = band.BandModel(device=dev)
    model.load(os.path.join(os.path.dirname(pa.__file__), "data", "band_model.npz"))
    for d in (workloads.config5(seed=91, n_pairs=512, strata=(0.4, 0.4, 0.2)),
              workloads.config4(seed=92, n_pairs=1024)):
        n = len(d["off1"]) - 1
        base = dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                    gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                    last_column_free=False, last_row_free=False, band_mode=0)
        plain = Aligner(base).compute_arrays(d["seq1"], d["off1"], d["seq2"], d["off2"])
        al = Aligner({**base, "band_mode": 1})
        model.to_context(al.context)
        tens = [torch.from_numpy(np.array(d["seq1"])).to(dev), torch.from_numpy(d["off1"].astype(np.int64)).to(dev),
                torch.from_numpy(np.array(d["seq2"])).to(dev), torch.from_numpy(d["off2"].astype(np.int64)).to(dev)]
        stream = torch.cuda.Stream(device=dev)
        for _ in range(2):
            out = torch.full((n * 16,), 0xCD, dtype=torch.uint8, device=dev)
            al.compute_device(*tens, out, stream=stream)
            torch.cuda.synchronize()
            got = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)
            for f in ("score", "end1", "end2"):
                assert np.array_equal(got[f], plain[f]), f
            assert ((got["flags"] & (BANDED | FULL | TRIVIAL)) != 0).all()

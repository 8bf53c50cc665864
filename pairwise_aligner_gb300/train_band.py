"""Train and evaluate the band predictor of band_mode 1 (global alignment).

    python -m pairwise_aligner_gb300.train_band --out pairwise_aligner_gb300/data/band_model.npz \
        --report band_report.json

Training data: seeded synthetic pairs from the learned-band workload (64-512 bp,
15/2/2 % divergence plus one or two 50-500 bp structural indels) and, so that
the predictor also covers long reads, the two long strata of the mixed stream
(1-10 kb at 8 %, 20-50 kb at 6 % plus structural indels).  Every pair is
labelled by the full GPU DP: the optimal-path diagonals at 8 checkpoint
columns (pa_band_labels) and the optimal score (pa_align_batch); inputs are the
12-mer diagonal histograms (pa_band_features_device).  The network is trained
with this package's own kernels (BandModel).

Evaluation on held-out seeds: the plain full DP, band_mode 1 (learned band) and
band_mode 2 (straight band, the same certificate and doubling without the
network) on the same pairs; scores must agree bit for bit.  Reported: the
certificate pass rate, the doubling rounds, the cells the banded DP computed,
and effective GCUPS (all m*n cells / wall time).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import band, workloads
from .aligner import RESULT_DTYPE, Aligner, Context

BANDED, FULL, TRIVIAL = 0x02, 0x04, 0x08


def global_config(d: dict, band_mode: int = 0) -> dict:
    return dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                last_column_free=False, last_row_free=False, band_mode=band_mode)


def training_set(n_short: int, n_long: int, seed: int) -> dict:
    parts = []
    for k in range(0, n_short, 262144):                 # config-4 generator, in seeded blocks
        parts.append(workloads.config4(seed=seed * 1000 + k // 262144, n_pairs=min(262144, n_short - k)))
    if n_long:
        d5 = workloads.config5(seed=seed * 1000 + 999, n_pairs=n_long, strata=(0.0, 0.9, 0.1))
        parts.append(d5)
    return workloads.concat(parts)


def _device(d: dict, dev):
    import torch
    return (torch.from_numpy(np.ascontiguousarray(d["seq1"])).to(dev),
            torch.from_numpy(d["off1"].astype(np.int64)).to(dev),
            torch.from_numpy(np.ascontiguousarray(d["seq2"])).to(dev),
            torch.from_numpy(d["off2"].astype(np.int64)).to(dev))


def label(d: dict, ctx: Context, chunk: int = 200000, log=print):
    """Inputs (n, 130) float32 on the device, targets (n, 9), mask (n,) -- all from the GPU DP."""
    import torch
    al = Aligner(global_config(d), context=ctx)
    cfg = al.c_config()
    n = len(d["off1"]) - 1
    m = np.diff(d["off1"].astype(np.int64))
    nn = np.diff(d["off2"].astype(np.int64))
    labs = np.zeros((n, 8), np.int32)
    score = np.zeros(n, np.int64)
    dev = torch.device(f"cuda:{ctx.device}")
    feats = torch.zeros((n, band.FEAT), dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    for s in range(0, n, chunk):
        part = workloads.subset(d, np.arange(s, min(n, s + chunk)))
        labs[s:s + chunk] = band.labels(ctx, cfg, part["seq1"], part["off1"], part["seq2"], part["off2"])
        score[s:s + chunk] = al.compute_arrays(part["seq1"], part["off1"], part["seq2"], part["off2"])["score"]
        feats[s:s + chunk] = band.features(*_device(part, dev))
    torch.cuda.synchronize()
    log(f"labelled {n} pairs in {time.perf_counter() - t0:.1f} s")
    y = band.targets(labs, m, nn, score, max(d["match"], 0))
    mask = ((m >= 9) & (nn >= 1)).astype(np.float32)
    return feats, y, mask


def evaluate(model: band.BandModel, d: dict, ctx: Context, repeats: int = 3, log=print) -> dict:
    import torch
    dev = torch.device(f"cuda:{ctx.device}")
    model.to_context(ctx)
    tens = _device(d, dev)
    n = len(d["off1"]) - 1
    cells = workloads.cells(d)
    out = {"pairs": n, "cells": cells}
    results = {}
    for name, mode in (("plain", 0), ("learned", 1), ("straight", 2)):
        al = Aligner(global_config(d, mode), context=ctx)
        res = torch.zeros((n, 16), dtype=torch.uint8, device=dev)
        al.compute_device(*tens, res, stats=True)                   # warm-up (and graph capture)
        times = []
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            al.compute_device(*tens, res, stats=True)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        st = al.last_stats
        r = res.cpu().numpy().reshape(-1).view(RESULT_DTYPE)
        flags = r["flags"].astype(np.int64)
        rounds = r["band_rounds"].astype(np.int64)
        results[name] = r["score"]
        t = float(np.median(times))
        entry = {"seconds": t, "effective_gcups": cells / t / 1e9, "device_ms": st["device_ms"]}
        if mode:
            nontriv = n - int(st["pairs_trivial"])
            banded = flags & BANDED != 0
            entry.update(pass_rate=float(st["pairs_banded"]) / max(nontriv, 1), pairs_banded=int(st["pairs_banded"]),
                         pairs_full_dp=int(st["pairs_full_dp"]), band_cells=int(st["band_cells"]),
                         band_cell_fraction=float(st["band_cells"]) / max(cells, 1),
                         rounds_tried=int(st["band_rounds"]),
                         rounds_histogram={int(k): int(v) for k, v in zip(*np.unique(rounds[banded], return_counts=True))})
        out[name] = entry
        log(f"{name}: {json.dumps(entry)}")
    out["bit_exact_learned"] = bool((results["learned"] == results["plain"]).all())
    out["bit_exact_straight"] = bool((results["straight"] == results["plain"]).all())
    out["speedup_learned"] = out["plain"]["seconds"] / out["learned"]["seconds"]
    out["speedup_straight"] = out["plain"]["seconds"] / out["straight"]["seconds"]
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train-pairs", type=int, default=2000000, help="learned-band workload pairs")
    ap.add_argument("--train-long", type=int, default=8000, help="long-read pairs (1-50 kb)")
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--eval-pairs", type=int, default=16384)
    ap.add_argument("--eval-mixed", type=int, default=32768, help="mixed-stream pairs (0: skip)")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "data", "band_model.npz"))
    ap.add_argument("--report", default=None)
    ap.add_argument("--load", default=None, help="evaluate these weights instead of training")
    a = ap.parse_args(argv)
    ctx = Context(0)
    model = band.BandModel(seed=a.seed, max_batch=a.batch)
    report = {"args": vars(a)}
    if a.load:
        model.load(a.load)
    else:
        t0 = time.perf_counter()
        d = training_set(a.train_pairs, a.train_long, a.seed)
        print(f"generated {len(d['off1']) - 1} training pairs in {time.perf_counter() - t0:.1f} s")
        x, y, mask = label(d, ctx)
        del d
        import torch
        t0 = time.perf_counter()
        hist = model.train(x.cpu().numpy(), y, mask, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, log=print)
        torch.cuda.synchronize()
        report["train"] = {"mse_per_epoch": hist, "seconds": time.perf_counter() - t0, "pairs": int(len(y))}
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        model.save(a.out)
    # held-out seeds: the learned-band workload and the mixed stream
    ev = workloads.config4(seed=424242, n_pairs=a.eval_pairs)
    report["config4_eval"] = evaluate(model, ev, ctx)
    if a.eval_mixed:
        ev5 = workloads.config5(seed=515151, n_pairs=a.eval_mixed)
        report["config5_eval"] = evaluate(model, ev5, ctx)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps({k: v for k, v in report.items() if k != "args"}, indent=1)[:4000])


if __name__ == "__main__":
    main()

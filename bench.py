#!/usr/bin/env python3
"""Throughput of the affine-gap score DP on GB300, in GCUPS (full m*n cells per second).

Workload: the local (Smith-Waterman-Gotoh) batch of 262,144 DNA pairs with
independent lengths uniform in 64..512, half related (15/2/2% mutations) and
half unrelated, scores +1/-4, gap_model_affine(-6, -1), score plus end
coordinates.  Synthetic and seeded (pairwise_aligner_gb300.workloads.config2).

One step = one call of the hot path over the whole batch:
  value  -- inputs already resident in HBM, pa_align_batch_device on one stream,
            CUDA events around K steps (inputs of ~150 MB plus ~300 MB of score
            tables exceed the 129 MB L2, so no flush is needed between steps);
  e2e    -- the same batch through pa_align_batch with pinned HOST buffers:
            host->device copies, the DP and the device->host result read per step.
  e2e_packed -- the same through pa_align_batch_packed: 2-bit packed host streams
            (a quarter of the sequence bytes cross to the device; DNA workloads).
  input_path -- GB/s of the 2-bit pack / unpack and rank-map kernels on 1 GiB.
  traceback -- with --traceback: GCUPS of pa_traceback_batch (alignment ops) on the batch.
  roofline -- the DP kernels' own duration (events inside the library) against
            the measured whole-chip rate of the cell-update instruction mix
            (pa_measure_roofline); HBM traffic against MEASURED_PEAKS.json.
  cpu_baseline -- the oracle's inter-sequence SIMD port on all host cores, on a
            bounded sample of the batch (rank 0 only).
  exact  -- after the timed region, every result of the batch (score and both end
            positions) compared with the scalar oracle on all host cores; the oracle is
            the checker here, never the thing timed (rank 0; a seeded sample when the
            batch is too large for the oracle to finish in about a minute).
  learned_band -- band mode 1 (the shipped predictor) against the plain full DP on the
            16,384 held-out pairs of the learned-band workload and on a 262,144-pair
            sample of the mixed global stream: GCUPS of both, certified pairs, band
            rounds, and whether the banded scores equal the plain ones.

--impl reference times the CPU implementation of the path (the reference's own
build when present, else the oracle's SIMD port) on the host cores.
N > 1 GPUs (torchrun): independent replicas, one full batch per rank, no
collective on the data path; value = all ranks' cells / max time.

--workload config1..config5 measures the other seeded workloads the same way
(config 3: 8,192 long reads; config 5: the 1,048,576-pair mixed stream), and
--band 1 / 2 runs global workloads in band mode (learned band with the shipped
predictor weights / straight band); scores are the same as --band 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "GCUPS (m*n cells/s), affine-gap local score DP + end coordinates, bit-exact"
METRIC_GLOBAL = "GCUPS (m*n cells/s), affine-gap global score DP, bit-exact"
WORKLOAD = "config2_local_262144_pairs_64-512bp_+1/-4/-6/-1"
BAND_MODEL = os.path.join(REPO, "pairwise_aligner_gb300", "data", "band_model.npz")
# DRAM bytes per cell of the short-pair local DP kernel (dp_short, 8 lanes per group, 32 rows
# per thread), from one ncu capture of its launch on all 262,144 pairs of this workload:
# dram__bytes.sum.per_second (207.49 GB/s) x gpu__time_duration.sum (4.95712 ms) over the
# launch's 2.1770e10 cells.  Most of it is the write-back of the 16-byte column slots.
DRAM_BYTES_PER_CELL = 207.492454e9 * 4.957120e-3 / 21769527988


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_workload(pairs: int | None, workload: str = "config2"):
    """The seeded workload; with PA_WORKLOAD_CACHE set, generated once per directory."""
    import numpy as np
    from pairwise_aligner_gb300 import workloads as W
    cache = os.environ.get("PA_WORKLOAD_CACHE")
    path = os.path.join(cache, f"{workload}_{pairs or 0}.npz") if cache else None
    if path and os.path.exists(path):
        z = np.load(path, allow_pickle=False)
        d = {k: z[k] for k in z.files}
        for k in ("local",):
            d[k] = bool(d[k])
        for k in ("match", "mismatch", "gap_open", "gap_extension", "config"):
            d[k] = int(d[k])
        d["name"] = str(d["name"])
        return d, W.cells(d)
    gen = W.GENERATORS[int(workload[-1])]
    d = gen() if not pairs else gen(n_pairs=pairs)
    if path:
        os.makedirs(cache, exist_ok=True)
        np.savez(path + ".tmp.npz", **{k: np.asarray(v) for k, v in d.items()})
        os.replace(path + ".tmp.npz", path)
    return d, W.cells(d)


def workload_name(d: dict, workload: str, n: int) -> str:
    if workload == "config2":
        return WORKLOAD
    return f"{d.get('name', workload)}_{n}_pairs_{d['match']:+d}/{d['mismatch']:+d}/{d['gap_open']:+d}/{d['gap_extension']:+d}"


def lanes_label(counts) -> str:
    """Which lane widths of the CPU port finished the sample's pairs."""
    return (f"pairs finished in 16 byte lanes: {counts[0]}, 8 int16 lanes: {counts[1]}, "
            f"4 int32 lanes: {counts[2]}")


PORT_LABEL = ("oracle inter-sequence SIMD port (oracle/pa_oracle.c, pa_oracle_bytes.cpp), 16-byte vectors, "
              "pthreads: local A/C/G/T pairs in 16 byte lanes (the reference's saturated int8 width), the "
              "rest in 8 int16 / 4 int32 lanes")


def cpu_sample_rate(d, budget_s: float, threads: int, counts=None):
    """Time the oracle's SIMD port on a leading sample of the batch sized to ~budget_s seconds."""
    import numpy as np
    from oracle import oracle as O
    from pairwise_aligner_gb300 import workloads as W
    cfg = O.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"], local=d["local"])
    n_total = len(d["off1"]) - 1
    n = min(n_total, 2048)
    while True:
        sub = W.subset(d, np.arange(n))
        t0 = time.perf_counter()
        O.simd_batch(cfg, sub["seq1"], sub["off1"], sub["seq2"], sub["off2"], nthreads=threads, counts=counts)
        dt = time.perf_counter() - t0
        if dt >= budget_s * 0.5 or n >= n_total:
            return W.cells(sub) / dt / 1e9, n, dt
        n = min(n_total, int(n * max(2.0, budget_s / max(dt, 1e-3))))


def reference_arm(args):
    import numpy as np
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import oracle as O
    from pairwise_aligner_gb300 import workloads as W
    d, _ = load_workload(args.pairs, args.workload)
    threads = os.cpu_count() or 1
    kind, label = "port", PORT_LABEL
    # one step = a bounded leading sample, sized so W + K steps take about two minutes
    per_step = max(0.5, min(5.0, 100.0 / max(1, args.steps + args.warmup)))
    rate, n, dt = cpu_sample_rate(d, per_step, threads)
    sub = W.subset(d, np.arange(n))
    cfg = O.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"], local=d["local"])
    for _ in range(args.warmup):
        O.simd_batch(cfg, sub["seq1"], sub["off1"], sub["seq2"], sub["off2"], nthreads=threads)
    times = []
    counts = [0, 0, 0]
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.simd_batch(cfg, sub["seq1"], sub["off1"], sub["seq2"], sub["off2"], nthreads=threads, counts=counts)
        times.append(time.perf_counter() - t0)
    cells = W.cells(sub)
    value = cells * len(times) / sum(times) / 1e9
    sample = f"first {n} of {len(d['off1']) - 1} pairs ({cells:.3g} cells) per step; {label}; {lanes_label(counts)}"
    line = {"impl": "reference", "metric": METRIC if d["local"] else METRIC_GLOBAL, "value": round(value, 3), "unit": "GCUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8 lanes (int16 / int32 where needed)",
            "data": "synthetic", "config": {"workload": workload_name(d, args.workload, len(d["off1"]) - 1),
                                            "pairs_per_step": n},
            "cpu_baseline": {"value": round(value, 3), "unit": "GCUPS", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def our_arm(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    import pairwise_aligner_gb300 as pa
    from pairwise_aligner_gb300.aligner import Aligner
    from pairwise_aligner_gb300 import build as B

    rank, world, local_rank = env_rank()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("gloo")
    B.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    d, cells = load_workload(args.pairs, args.workload)
    n = len(d["off1"]) - 1
    free = bool(d["local"])
    if args.band and d["local"]:
        raise SystemExit("--band applies to the global workloads (config1, config3, config4, config5)")
    conf = dict(local=d["local"], match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                gap_extension=d["gap_extension"], first_column_free=free, first_row_free=free,
                last_column_free=free, last_row_free=free, width_hint=0, band_mode=args.band)
    ctx = pa.Context(local_rank, group_threads=args.group_threads, kernel_variant=args.variant)
    if args.band == 1:
        from pairwise_aligner_gb300 import band as BD
        model = BD.BandModel(device=dev)
        model.load(BAND_MODEL)
        model.to_context(ctx)
    if args.band and args.band_margin > 0:
        ctx.set_band_options(margin=args.band_margin)
    al = Aligner(conf, device=local_rank, context=ctx)
    peak = ctx.roofline()

    s1 = torch.from_numpy(d["seq1"]).to(dev)
    s2 = torch.from_numpy(d["seq2"]).to(dev)
    o1 = torch.from_numpy(d["off1"].astype(np.int64)).to(dev)
    o2 = torch.from_numpy(d["off2"].astype(np.int64)).to(dev)
    out = torch.empty(n * 16, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    # warm-up (captures the CUDA graph), then K timed steps
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            al.compute_device(s1, o1, s2, o2, out, stream=stream)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    # inputs smaller than L2 (the small workloads): time every step alone, after an L2 flush
    small = int(d["off1"][-1] + d["off2"][-1]) * 3 + 16 * n < 129e6
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if small else None
    with ClockSampler(local_rank) as clk:
        time.sleep(0.3)
        if small:
            total = 0.0
            for _ in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                al.compute_device(s1, o1, s2, o2, out, stream=stream)
                b.record(stream)
                b.synchronize()
                total += a.elapsed_time(b)
            step_ms = total / args.steps
        else:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                al.compute_device(s1, o1, s2, o2, out, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms = e0.elapsed_time(e1) / args.steps
        time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    ms = max_over_ranks(step_ms, world)
    value = replica_throughput(cells, ms, world)

    # DP kernels alone (events inside the library, same stream), one call at a time
    dp = []
    for _ in range(max(3, min(args.steps, 5))):
        al.compute_device(s1, o1, s2, o2, out, stream=stream, stats=True)
        dp.append(al.last_stats["dp_ms"])
    st = al.last_stats
    dp_ms = statistics.mean(dp)
    launches_per_step = int(st["kernel_launches"])
    res = np.frombuffer(out.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE)

    # end to end through the host-buffer C ABI from pinned memory
    pin = {k: torch.from_numpy(np.ascontiguousarray(d[k])).pin_memory() for k in ("seq1", "off1", "seq2", "off2")}
    hs = {k: v.numpy() for k, v in pin.items()}
    res_pin = torch.empty(n * 16, dtype=torch.uint8).pin_memory().numpy().view(pa.RESULT_DTYPE)
    for _ in range(2):
        al.compute_arrays(hs["seq1"], hs["off1"], hs["seq2"], hs["off2"], stats=False, out=res_pin)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_res = al.compute_arrays(hs["seq1"], hs["off1"], hs["seq2"], hs["off2"], stats=False, out=res_pin)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    assert np.array_equal(host_res["score"], res["score"]), "host and device entry points disagree"
    h2d = int(sum(pin[k].numel() * pin[k].element_size() for k in pin))
    d2h = n * 16

    # the same through the 2-bit packed host entry (DNA workloads; the inputs are kept packed
    # on the host, so the packing happens before the timed region)
    e2e_packed = None
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    if np.isin(d["seq1"], acgt).all() and np.isin(d["seq2"], acgt).all():
        from pairwise_aligner_gb300 import seqio
        w1 = torch.from_numpy(seqio.pack_2bit(d["seq1"])[0]).pin_memory().numpy()
        w2 = torch.from_numpy(seqio.pack_2bit(d["seq2"])[0]).pin_memory().numpy()
        for _ in range(2):
            al.compute_packed(w1, hs["off1"], w2, hs["off2"], stats=False, out=res_pin)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            packed_res = al.compute_packed(w1, hs["off1"], w2, hs["off2"], stats=False, out=res_pin)
        pk_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
        assert np.array_equal(packed_res["score"], res["score"]), "packed and byte entry points disagree"
        e2e_packed = {"value": round(replica_throughput(cells, pk_s * 1e3, world), 2), "unit": "GCUPS",
                      "h2d_bytes_per_step": int(w1.nbytes + w2.nbytes + pin["off1"].numel() * 8 +
                                                pin["off2"].numel() * 8),
                      "d2h_bytes_per_step": d2h, "entry": "pa_align_batch_packed (2-bit host streams)"}
    input_path = input_kernels(dev, stream, ctx) if not args.no_input else None

    # the traceback path (alignment ops) over the same batch, host buffers, checked against
    # the score-only results
    traceback = None
    if args.traceback:
        tb_res = None
        al.compute_traceback_arrays(hs["seq1"], hs["off1"], hs["seq2"], hs["off2"])
        dev_ms, t0 = [], time.perf_counter()
        for _ in range(args.steps):
            tb_res, tb_aln, _, _ = al.compute_traceback_arrays(hs["seq1"], hs["off1"], hs["seq2"], hs["off2"])
            dev_ms.append(al.last_stats["device_ms"])
        tb_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
        assert np.array_equal(tb_res["score"], res["score"]), "traceback and score-only results disagree"
        traceback = {"value": round(replica_throughput(cells, tb_s * 1e3, world), 2), "unit": "GCUPS",
                     "device_gcups": round(cells / (statistics.mean(dev_ms) * 1e-3) / 1e9, 2),
                     "ms_per_step": round(tb_s * 1e3, 3), "mean_ops": round(float(tb_aln["n_ops"].mean()), 2),
                     "entry": "pa_traceback_batch (host buffers; score, end, begin and ops of every pair)"}

    achieved = cells / (dp_ms * 1e-3) / 1e9
    peak_gcups = peak["s16x2_cells_per_s"] / 1e9
    alg_bytes = int(d["off1"][-1] + d["off2"][-1]) + 16 * n          # inputs read + results written
    line = {
        "metric": METRIC if d["local"] else METRIC_GLOBAL, "value": round(value, 2), "unit": "GCUPS",
        "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16x2 lanes (int32 where a pair needs it)", "data": "synthetic",
        "config": {"workload": workload_name(d, args.workload, n), "pairs": n, "cells": cells,
                   "group_threads": ctx_G(args), "band_mode": args.band,
                   "l2": ("inputs (sequence bytes, per-column slots or score tables) larger than the 129 MB L2; no flush" if not small
                          else "inputs smaller than L2: a 256 MB buffer is written before every timed step"),
                   "pairs_s16": st["pairs_s16"], "pairs_s32": st["pairs_s32"], "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(replica_throughput(cells, e2e_s * 1e3, world), 2), "unit": "GCUPS",
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "int_dpx", "achieved": round(achieved, 1), "peak": round(peak_gcups, 1),
                     "unit": "GCUPS", "frac": round(achieved / peak_gcups, 4),
                     "traffic": int(DRAM_BYTES_PER_CELL * cells) if args.workload == "config2" else None,
                     "peak_source": "pa_measure_roofline: whole-chip s16x2 cell-update instruction mix, measured live",
                     "kernel": "the DP kernels of one call (config 2: dp_short, s16x2, 8 lanes per group, "
                               "32 rows per thread)", "kernel_ms": round(dp_ms, 4),
                     "local_mix": ({"peak": round(peak["s16x2_local_cells_per_s"] / 1e9, 1),
                                    "frac": round(achieved / (peak["s16x2_local_cells_per_s"] / 1e9), 4),
                                    "note": "the same mix plus local scoring's per-column maximum "
                                            "(k_roofline<L16, TRACK>), for context; frac above is the one "
                                            "against the recurrence alone"}
                                   if d["local"] and peak.get("s16x2_local_cells_per_s") else None),
                     "hbm": {"achieved": round(alg_bytes / (dp_ms * 1e-3) / 1e9, 1),
                             "peak": hbm_peak(), "unit": "GB/s",
                             "frac": round(alg_bytes / (dp_ms * 1e-3) / 1e9 / hbm_peak(), 5)}},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
    }
    if e2e_packed:
        line["e2e_packed"] = e2e_packed
    if input_path:
        line["input_path"] = input_path
    if traceback:
        line["traceback"] = traceback
    if args.band:
        line["band"] = {k: st[k] for k in ("pairs_banded", "pairs_full_dp", "band_cells", "band_rounds")}
        line["band"]["options"] = ctx.band_options()
    if rank == 0 and not args.no_exact:
        line["exact"] = check_exact(d, res)
    if rank == 0 and world == 1 and args.workload == "config2" and not args.no_band_section:
        line["learned_band"] = learned_band_section(dev, stream, args)
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        counts = [0, 0, 0]
        rate, npairs, dt = cpu_sample_rate(d, args.cpu_seconds, threads, counts)
        line["cpu_baseline"] = {"value": round(rate, 3), "unit": "GCUPS", "cores": threads, "kind": "port",
                                "sample": f"first {npairs} pairs of the batch, {dt:.1f} s; {PORT_LABEL}; "
                                          f"{lanes_label(counts)}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def check_exact(d: dict, res) -> dict:
    """Every result of the batch against the scalar oracle (the checker, outside any timed
    region): when the batch holds more than 3e10 cells, a seeded sample of 4,096 pairs."""
    import numpy as np
    from oracle import oracle as O
    from pairwise_aligner_gb300 import workloads as W
    n = len(d["off1"]) - 1
    idx = np.arange(n)
    if W.cells(d) > 3e10:
        idx = np.sort(np.random.default_rng(99).choice(n, size=min(n, 4096), replace=False))
    sub = W.subset(d, idx) if len(idx) < n else d
    free = bool(d["local"])
    oc = O.make_cfg(d["match"], d["mismatch"], d["gap_open"], d["gap_extension"], local=d["local"],
                    first_column_free=free, first_row_free=free, last_column_free=free, last_row_free=free)
    t0 = time.perf_counter()
    sc, e1, e2 = O.align_batch(oc, sub["seq1"], sub["off1"], sub["seq2"], sub["off2"], nthreads=os.cpu_count())
    r = res[idx]
    same = bool(np.array_equal(r["score"], sc) and np.array_equal(r["end1"], e1) and np.array_equal(r["end2"], e2))
    return {"equal": same, "pairs_checked": int(len(idx)), "of_pairs": int(n),
            "against": "scalar oracle (oracle/pa_oracle.c), score + end1 + end2",
            "seconds": round(time.perf_counter() - t0, 1)}


def learned_band_section(dev, stream, args) -> dict:
    """Band mode 1 with the shipped predictor against the plain DP on two global workloads."""
    import numpy as np
    import torch
    import pairwise_aligner_gb300 as pa
    from pairwise_aligner_gb300 import band as BD
    from pairwise_aligner_gb300 import workloads as W
    from pairwise_aligner_gb300.aligner import Aligner
    out = {"model": "pairwise_aligner_gb300/data/band_model.npz", "unit": "GCUPS (full m*n cells per second)"}
    model = BD.BandModel(device=dev)
    model.load(BAND_MODEL)
    for name, d in (("config4_eval_16384_pairs", W.config4(seed=424242, n_pairs=16384)),
                    ("config5_sample_262144_pairs", W.config5(seed=515151, n_pairs=262144))):
        cells = W.cells(d)
        n = len(d["off1"]) - 1
        s1 = torch.from_numpy(d["seq1"]).to(dev)
        s2 = torch.from_numpy(d["seq2"]).to(dev)
        o1 = torch.from_numpy(d["off1"].astype(np.int64)).to(dev)
        o2 = torch.from_numpy(d["off2"].astype(np.int64)).to(dev)
        entry = {"pairs": n, "cells": cells}
        results = {}
        for mode in (0, 1):
            ctx = pa.Context(dev.index or 0)
            if mode == 1:
                model.to_context(ctx)
            conf = dict(local=False, match=d["match"], mismatch=d["mismatch"], gap_open=d["gap_open"],
                        gap_extension=d["gap_extension"], first_column_free=False, first_row_free=False,
                        last_column_free=False, last_row_free=False, width_hint=0, band_mode=mode)
            al = Aligner(conf, context=ctx)
            out_t = torch.empty(n * 16, dtype=torch.uint8, device=dev)
            for _ in range(2):
                al.compute_device(s1, o1, s2, o2, out_t, stream=stream, stats=True)
            torch.cuda.synchronize()
            steps = 3
            flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
            total = 0.0
            for _ in range(steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                al.compute_device(s1, o1, s2, o2, out_t, stream=stream)
                b.record(stream)
                b.synchronize()
                total += a.elapsed_time(b)
            ms = total / steps
            results[mode] = np.frombuffer(out_t.cpu().numpy().tobytes(), dtype=pa.RESULT_DTYPE).copy()
            key = "plain" if mode == 0 else "band"
            entry[key] = {"gcups": round(cells / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 3)}
            if mode == 1:                         # the counters, from one more (untimed) call
                al.compute_device(s1, o1, s2, o2, out_t, stream=stream, stats=True)
                st = al.last_stats
                entry[key].update(certified_pairs=int(st["pairs_banded"]), full_dp_pairs=int(st["pairs_full_dp"]),
                                  band_cells=int(st["band_cells"]), rounds=int(st["band_rounds"]))
            ctx.close()
            del flush
        entry["band_over_plain"] = round(entry["band"]["gcups"] / entry["plain"]["gcups"], 3)
        entry["exact"] = bool(np.array_equal(results[0]["score"], results[1]["score"]))
        out[name] = entry
        del s1, s2, o1, o2
    torch.cuda.empty_cache()
    return out


def input_kernels(dev, stream, ctx, n: int = 1 << 30, reps: int = 5) -> dict:
    """GB/s of the input-path kernels on 1 GiB of bytes (inputs and outputs well beyond L2):
    algorithmic bytes = bytes read + bytes written once."""
    import torch
    from pairwise_aligner_gb300 import seqio
    g = torch.Generator(device=dev).manual_seed(5)
    codes = torch.randint(0, 4, (n,), device=dev, dtype=torch.uint8, generator=g)
    letters = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=dev)[codes.long()]
    del codes
    words = torch.empty((n + 15) // 16, dtype=torch.int32, device=dev)
    back = torch.empty(n, dtype=torch.uint8, device=dev)
    ranks = torch.empty(n, dtype=torch.int8, device=dev)
    out = {}
    jobs = {"pack_2bit": (lambda: seqio.pack_2bit_device(ctx, letters, words), n + n // 4),
            "unpack_2bit": (lambda: seqio.unpack_2bit_device(ctx, words, 0, n, back), n // 4 + n),
            "rank_map": (lambda: seqio.rank_map_device(ctx, b"ACGTN", letters, ranks), 2 * n)}
    peak = hbm_peak()
    stream.wait_stream(torch.cuda.current_stream())          # the inputs were made on torch's stream
    with torch.cuda.stream(stream):
        for name, (fn, nbytes) in jobs.items():
            fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b) / reps
            gbs = nbytes / (ms * 1e-3) / 1e9
            out[name] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}
    torch.cuda.synchronize()
    assert torch.equal(back, letters), "unpack(pack(x)) != x"
    out.update({"bytes": n, "peak_gbs": peak, "unit": "GB/s (algorithmic bytes read + written)"})
    del letters, words, back, ranks
    torch.cuda.empty_cache()
    return out


def max_over_ranks(x: float, world: int) -> float:
    """The slowest rank's value: a job's time is its slowest rank's."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells_per_rank: int, ms_per_step: float, world: int) -> float:
    """Whole-job GCUPS of N independent replicas: every rank's cells over the slowest time."""
    return cells_per_rank * world / (ms_per_step * 1e-3) / 1e9


def hbm_peak() -> float:
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0          # fallback figure of the profiling recipe


def ctx_G(args):
    return args.group_threads or 8


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--pairs", type=int, default=0, help="override the batch size (default: 262,144)")
    ap.add_argument("--group-threads", type=int, default=0)
    ap.add_argument("--variant", type=int, default=-1)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-input", action="store_true", help="skip the input-path kernel measurement")
    ap.add_argument("--no-exact", action="store_true", help="skip the oracle check of the batch's results")
    ap.add_argument("--no-band-section", action="store_true", help="skip the learned-band comparison")
    ap.add_argument("--traceback", action="store_true", help="also time pa_traceback_batch on the batch")
    ap.add_argument("--workload", choices=["config1", "config2", "config3", "config4", "config5"], default="config2")
    ap.add_argument("--band", type=int, choices=[0, 1, 2], default=0,
                    help="band mode for global workloads: 1 learned (shipped weights), 2 straight")
    ap.add_argument("--band-margin", type=float, default=0.0, help="band mode: start-width margin (default 1.25)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    return reference_arm(args) if args.impl == "reference" else our_arm(args)


if __name__ == "__main__":
    sys.exit(main())

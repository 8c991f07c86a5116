"""Benchmark: FFA acceleration search, 2^23 samples, on one GB300 (or N replicas).

Workload (one step): the full time-domain FFA search of one float32 series of
2^23 samples at 64 us (noise N(0,1) plus a 5 ms pulsar with 20 m/s^2
line-of-sight acceleration at S/N 15): frequency 50-500 Hz, acceleration
+-50 m/s^2, 64 bins, boxcar widths 1,2,4,8,16. Brute fold, 9 DP levels, the
last two banded and fused with boxcar scoring; 193 x 7,730,942 final
parameter sets = 1.49e9 period-trials, every one scored at every width.

``value``   period-trials/s with the series already in HBM (CUDA events).
``e2e``     the same through ``ffa_search`` from pinned host buffers: the H2D
            copy of the series and the D2H read of the best candidate are
            inside the timed region (wall clock, synchronised).
``--impl reference`` times the CPU oracle (the C restatement of pyloki's numba
loops, all host threads) on a bounded frequency band of the same search.

Under torchrun every rank searches its own series (independent replicas,
weak scaling); the step time is the max over ranks.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
# the batched pruning runs put many streams of small kernels in flight: give
# each of them its own hardware queue (a per-process setting, read at CUDA
# initialisation)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "period-trials/s"
WORKLOAD = "ffa_accel_search_2^23"
# DRAM bytes (read + write) per final trial of the fused last two levels:
# ncu capture of one launch of the same search at 2^21 samples (13 x 1932736
# trials); profiles/ffa_final_tiled64_kernel_ffa_accel_2^21.md. The banded
# path's figure comes from three full-band launches at 2^21
# (profiles/band_union64_kernel_ffa_accel_2^21.md).
FINAL_DRAM_BYTES_PER_TRIAL = {"tiled": 70.2, "banded": 259.0}
FINAL_KERNEL = {"tiled": "ffa_final_tiled64_kernel (last two levels fused per tile: "
                         "penultimate rows built in shared memory, lane-per-trial scoring)",
                "banded": "band_union64_kernel (penultimate band + fused final-level scoring)",
                "level": "ffa_level_score_kernel (final level fused with scoring)"}
BF16_TOP = 64        # candidates re-scored in FP64 and checked against the FP64 oracle
BF16_SAMPLE = 192    # random trials added to the FP64 error sample
BATCH_WORKLOAD = "ffa_jerk_batch_2^20-2^23"
BATCH_SERIES = 32    # bounded sample of the 256-series batch (first series of the draw)
BATCH_K = 16         # candidates kept per series


def make_cfg(freq_lo: float = 50.0, freq_hi: float = 500.0, nsamps: int = 2**23,
             use_fourier: bool = False):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig

    return PulsarSearchConfig(
        nsamps=nsamps, tsamp=64e-6, nbins=64, eta=1.0,
        param_limits=ParamLimits.from_taylor((freq_lo, freq_hi), accel=(-50.0, 50.0)).limits,
        ducy_max=0.25, wtsp=2.0, use_fourier=use_fourier, bseg_brute=16384)


def make_series(seed: int):
    from pyloki_gb300.simulation import make_series as ms

    return ms(2**23, 64e-6, freq=200.0, snr=15.0, ducy=0.05, accel=20.0, seed=seed)


def cpu_band_cfg(band_hz: float):
    """The same search restricted to [500 - band_hz, 500] Hz: identical bseg,
    frequency step and acceleration grid (the grids depend on f_max only)."""
    return make_cfg(500.0 - band_hz, 500.0)


PRUNE_WORKLOAD = "taylor4_prune_circular_orbit_2^22"
PRUNE_MAX_SUGG = 2**18
PRUNE_MULTI_RUNS = 64   # reference segments of the multi-run measurement
PRUNE_WORKERS = 4      # concurrent runs (host threads and CUDA streams)
PRUNE_STREAMS = 16     # concurrent device-resident runs (CUDA streams, one host thread)
PRUNE_BATCH = 1024
PRUNE_SCHEME = ROOT / "tests" / "golden" / "prune_scheme_taylor4.npz"
PRUNE_SCHEME_NOTE = "designed (DynamicThresholdScheme, least-cost path at 90% of S/N 10)"
# HBM bytes per leaf of prune_score_kernel: the parent fold (2 x 64 f32) read
# once, the score (f32), grid indices (2 x i32) and phase (f64) written. The
# added segment's fold (146 rows, 75 KB) stays in L2.
PRUNE_SCORE_BYTES_PER_LEAF = 2 * 64 * 4 + 4 + 8 + 8


def make_prune_cfg(circular: bool = False, fourier: bool = False):
    """Circular-orbit search with a Taylor tree to the 4th derivative: 2^22
    samples at 64 us, 128 segments, 64 bins, FFA grid (1, 1, 1, 146). With
    ``circular``, the circular-orbit tree of order 5 on the same series (FFA
    grid (1, 1, 1, 1, 146), P_orb_min 2 h); with ``fourier``, the FFA and the
    tree over complex (Fourier-domain) folds, the reference's default."""
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig

    n = 2**22
    order = 5 if circular else 4
    lim = ParamLimits.from_circular(333.33, p_orb_min=7200.0, poly_order=order)
    return PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
                              param_limits=lim.limits, use_fourier=fourier, bseg_ffa=n // 128,
                              prune_poly_order=order, p_orb_min=7200.0 if circular else 0.0)


def make_prune_series(seed: int):
    """3 ms pulsar (S/N 10) in a circular orbit: P_orb 2-10 h, projected
    semi-major axis 0.1-2 lt-s, orbital phase uniform; all drawn from ``seed``."""
    from pyloki_gb300.simulation import make_series as ms

    rng = np.random.default_rng(seed)
    orbit = (rng.uniform(2.0, 10.0) * 3600.0, rng.uniform(0.1, 2.0), rng.uniform(0, 2 * np.pi))
    return ms(2**22, 64e-6, freq=333.33, snr=10.0, orbit=orbit, seed=seed), orbit


def prune_thresholds(nseg: int) -> np.ndarray:
    """The designed per-level thresholds of the pruning workload: the
    reference's threshold-design workflow (DynamicThresholdScheme over the
    tree's branching pattern, least-cost path keeping 90 % of S/N-10 signals,
    rounded to 0.1), made by tests/golden/make_prune_scheme.py."""
    with np.load(PRUNE_SCHEME) as d:
        thr = d["thresholds"].astype(np.float64)
    if len(thr) != nseg - 1:
        msg = f"the threshold scheme has {len(thr)} levels, the search {nseg - 1}"
        raise ValueError(msg)
    return thr


def prune_cpu(nthreads: int = 0, circular: bool = False) -> dict:
    """The same pruning run on the CPU oracle (all host threads); with
    ``circular``, the circular-orbit tree of order 5."""
    from oracle import oracle as O
    from oracle.prune_oracle import PruneRun

    cfg = make_prune_cfg(circular=circular)
    ts, _ = make_prune_series(seed=2000)
    fold = O.ffa_execute(ts.ts_e, ts.ts_v, cfg, nthreads)
    n = cfg.niters_ffa
    nseg = fold.shape[0]
    run = PruneRun(cfg, fold, cfg.get_param_arr(cfg.get_dparams(n)), cfg.get_dparams_actual(n),
                   prune_thresholds(nseg), max_sugg=PRUNE_MAX_SUGG, batch_size=PRUNE_BATCH,
                   nthreads=nthreads)
    dt = run.run(nseg // 2)
    return {"value": run.n_leaves_total / dt, "unit": "leaves/s", "cores": O.max_threads(),
            "kind": "port", "leaves": run.n_leaves_total, "seconds": dt,
            "sample": f"one full run ({nseg - 1} levels, ref segment {nseg // 2})"}


def bench_prune_gpu(args, dev) -> dict:
    """Prune leaves/s of the pruning workload run from PRUNE_MULTI_RUNS
    reference segments per step (prune_dyp_tree's n_runs), batched: every run
    device-resident in its own CUDA graph, PRUNE_STREAMS runs at once on
    their own streams. Beside it: one run device-resident, one run level by
    level (the plain path), and the batched job end to end from a pinned host
    series."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBatch, PruneBlockBatch, Pruning
    from pyloki_gb300.timeseries import TimeSeries

    from pyloki_gb300 import _lib

    lib = _lib.load()
    cfg = make_prune_cfg()
    ts_host, orbit = make_prune_series(seed=2000)
    e_pin = torch.from_numpy(ts_host.ts_e).pin_memory()
    v_pin = torch.from_numpy(ts_host.ts_v).pin_memory()
    dyp = DynamicProgramming(TimeSeries(e_pin.to(dev), v_pin.to(dev), cfg.tsamp), cfg,
                             device=dev)
    dyp.initialize()
    dyp.execute()
    nseg = dyp.nsegments
    thr = prune_thresholds(nseg)
    ref = nseg // 2
    refs = [int(r) for r in np.linspace(4, nseg - 5, args.prune_runs).round()]
    kw = {"max_sugg": PRUNE_MAX_SUGG, "batch_size": PRUNE_BATCH}
    prn = Pruning(dyp, thr, **kw)

    def level_run(events=None) -> int:
        """The plain path: level by level, one host wait per level for the
        child count and one for the survivor count."""
        prn.score_events = events
        prn.initialize(ref)
        for _ in range(nseg - 1):
            prn.execute_iter()
            if prn.prune_complete:
                break
        prn._do_ascend()
        return sum(st.n_leaves for st in prn.pstats[1:])

    def device_run() -> int:
        """One run device-resident: every level in one CUDA graph."""
        prn.run_device(ref, graph=True)
        prn._do_ascend()
        return sum(st.n_leaves for st in prn.pstats[1:])

    runner = PruneBlockBatch(thr, **kw)
    streams = PruneBatch(thr, n_streams=args.prune_streams, **kw)

    def batched(d=dyp) -> int:
        """Every run at once: one launch per step of a level over all runs,
        the kernels replayed from one CUDA graph."""
        res = runner.run([(d, r) for r in refs])
        return sum(st.n_leaves for r in res for st in r["level_stats"][1:])

    def batched_streams(d=dyp) -> int:
        """Every run device-resident in its own graph, several at once on
        their own streams."""
        res = streams.run([(d, r) for r in refs])
        return sum(st.n_leaves for r in res for st in r["level_stats"][1:])

    def timed(fn, steps):
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        n = sum(fn() for _ in range(steps))
        e1.record()
        torch.cuda.synchronize(dev)
        return n, e0.elapsed_time(e1)

    for _ in range(args.warmup):
        level_run()
        device_run()
        batched()
        batched_streams()
    # kernels per step, counted on an uncaptured step (a graph replay does
    # not pass through the library's launch counter)
    runner._graphs.clear()
    runner._seen.clear()
    c0 = lib.loki_launch_count()
    batched()
    step_launches = lib.loki_launch_count() - c0
    batched()  # captures the graph again
    with ClockSampler(dev.index) as clocks:
        leaves, ms = timed(batched, args.steps)
    streams_leaves, streams_ms = timed(batched_streams, args.steps)
    single_leaves, single_ms = timed(device_run, args.steps)
    plain_leaves, plain_ms = timed(level_run, args.steps)
    # the score kernel's own time for the roofline: one more batched step,
    # uncaptured, with CUDA events around every level's score launch (all
    # runs in one launch), outside the timed steps
    runner.time_score = True
    res = runner.run([(dyp, r) for r in refs])
    runner.time_score = False
    score_ms = float(runner.score_ms.sum())
    score_leaves = sum(st.n_leaves for r in res for st in r["level_stats"][1:])
    score_launches = int(runner.score_ms.size)
    peak, peak_kind = measured_peak_hbm()
    achieved = score_leaves * PRUNE_SCORE_BYTES_PER_LEAF / (score_ms * 1e-3) / 1e9
    value = leaves / (ms * 1e-3)
    plain_value = plain_leaves / (plain_ms * 1e-3)

    # end to end: pinned host series -> FFA -> the batched runs -> results on
    # the host (every run's surviving parameters and scores)
    from pyloki_gb300.timeseries import TimeSeries as TS

    host_ts = TS(e_pin, v_pin, cfg.tsamp)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e2e_leaves = 0
    d2h = 0
    for _ in range(args.steps):
        dp = DynamicProgramming(host_ts, cfg, device=dev)
        dp.initialize()
        dp.execute()
        res = runner.run([(dp, r) for r in refs])  # graphs rebound to the new fold
        e2e_leaves += sum(st.n_leaves for r in res for st in r["level_stats"][1:])
        d2h = sum(r["param_sets"].nbytes + r["scores"].nbytes + r["scores_ep"].nbytes
                  for r in res)
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    return {
        "metric": "prune leaves/s", "value": value, "unit": "leaves/s",
        "path": (f"batched: {len(refs)} reference segments per step, every step of a level "
                 f"one launch over all runs (loki_prune_run_batch), replayed from one CUDA "
                 f"graph; seeds, ascend and read-back one launch each"),
        "ms_per_step": ms / args.steps, "leaves_per_step": leaves // args.steps,
        "streams": {"value": streams_leaves / (streams_ms * 1e-3),
                    "ms_per_step": streams_ms / args.steps,
                    "note": (f"each run device-resident in its own CUDA graph, "
                             f"{args.prune_streams} runs at once on their own streams")},
        "single_run": {"value": single_leaves / (single_ms * 1e-3),
                       "ms_per_run": single_ms / args.steps,
                       "leaves_per_run": single_leaves // args.steps,
                       "note": "one run (reference segment 64) device-resident, one graph"},
        "plain": {"value": plain_value, "ms_per_run": plain_ms / args.steps,
                  "leaves_per_run": plain_leaves // args.steps,
                  "note": "one run level by level with two host waits per level"},
        "speedup_vs_plain": value / plain_value,
        "dtype": "f32 folds, f64 parameters",
        "data": "synthetic (seeded N(0,1) noise + 3 ms pulsar in a circular orbit, S/N 10)",
        "config": {"workload": PRUNE_WORKLOAD, "nsamps": cfg.nsamps, "tsamp": cfg.tsamp,
                   "nbins": cfg.nbins, "poly_order": 4, "segments": nseg,
                   "ffa_grid": cfg.get_param_grid_count(cfg.niters_ffa).tolist(),
                   "widths": cfg.score_widths.tolist(), "max_sugg": PRUNE_MAX_SUGG,
                   "batch_size": PRUNE_BATCH, "ref_segments": len(refs),
                   "driver": "level-synchronous batch (loki_prune_run_batch)",
                   "thresholds": PRUNE_SCHEME_NOTE,
                   "orbit": {"p_orb_h": orbit[0] / 3600, "x_lts": orbit[1], "psi": orbit[2]},
                   "l2": "segment folds (75 KB) are L2-resident; tree folds stream"},
        "roofline": {"kernel": "bj_score_kernel (resolve + gather + shift-add + score, "
                               "every run of the step in one launch per level)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_per_leaf": PRUNE_SCORE_BYTES_PER_LEAF,
                     "kernel_ms_per_step": score_ms,
                     "launches_per_step": score_launches, "traffic": None},
        "e2e": {"value": e2e_leaves / e2e_s, "unit": "leaves/s",
                "ms_per_step": e2e_s * 1e3 / args.steps, "h2d_bytes_per_step": 8 * cfg.nsamps,
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": step_launches * args.steps,
        "clocks": clocks.summary(),
        "survivors": int(prn.world_tree.valid_size),
    }


def bench_prune_fourier(args, dev) -> dict:
    """The pruning step over complex (Fourier-domain) folds, the reference's
    default mode: the same series, thresholds and reference segments, every
    run level-synchronously in the batch; beside it one run level by level."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBlockBatch, Pruning

    cfg = make_prune_cfg(fourier=True)
    ts, _ = make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=dev)
    dyp.initialize()
    dyp.execute()
    nseg = dyp.nsegments
    thr = prune_thresholds(nseg)
    refs = [int(r) for r in np.linspace(4, nseg - 5, args.prune_runs).round()]
    kw = {"max_sugg": PRUNE_MAX_SUGG, "batch_size": PRUNE_BATCH}
    runner = PruneBlockBatch(thr, **kw)
    prn = Pruning(dyp, thr, **kw)

    def batched() -> int:
        res = runner.run([(dyp, r) for r in refs])
        return sum(st.n_leaves for r in res for st in r["level_stats"][1:])

    def level_run() -> int:
        prn.initialize(nseg // 2)
        for _ in range(nseg - 1):
            prn.execute_iter()
            if prn.prune_complete:
                break
        prn._do_ascend()
        return sum(st.n_leaves for st in prn.pstats[1:])

    def timed(fn, steps):
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        n = sum(fn() for _ in range(steps))
        e1.record()
        torch.cuda.synchronize(dev)
        return n, e0.elapsed_time(e1)

    for _ in range(2):  # uncaptured, then captured
        batched()
    level_run()
    steps = max(1, min(args.steps, 3))
    leaves, ms = timed(batched, steps)
    plain_leaves, plain_ms = timed(level_run, 1)
    return {"metric": "prune leaves/s (complex folds)", "value": leaves / (ms * 1e-3),
            "unit": "leaves/s", "ms_per_step": ms / steps, "leaves_per_step": leaves // steps,
            "plain": {"value": plain_leaves / (plain_ms * 1e-3), "ms_per_run": plain_ms,
                      "leaves_per_run": plain_leaves},
            "config": {"workload": PRUNE_WORKLOAD.replace("prune", "prune_fourier"),
                       "ref_segments": len(refs), "fold": "complex64, nbins // 2 + 1",
                       "driver": "level-synchronous batch (loki_prune_run_batch, fourier)"}}


def bench_prune_circ(args, dev) -> dict:
    """The pruning step of the circular-orbit tree (order 5, crackle added)
    on the same series and thresholds: every run level-synchronously in the
    batch; beside it the same runs each device-resident in its own CUDA
    graph on several streams."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBatch, PruneBlockBatch

    cfg = make_prune_cfg(circular=True)
    ts, _ = make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=dev)
    dyp.initialize()
    dyp.execute()
    nseg = dyp.nsegments
    thr = prune_thresholds(nseg)
    refs = [int(r) for r in np.linspace(4, nseg - 5, args.prune_runs).round()]
    kw = {"max_sugg": PRUNE_MAX_SUGG, "batch_size": PRUNE_BATCH}
    runner = PruneBlockBatch(thr, **kw)
    streams = PruneBatch(thr, n_streams=args.prune_streams, **kw)

    def batched() -> int:
        res = runner.run([(dyp, r) for r in refs])
        return sum(st.n_leaves for r in res for st in r["level_stats"][1:])

    def batched_streams() -> int:
        res = streams.run([(dyp, r) for r in refs])
        return sum(st.n_leaves for r in res for st in r["level_stats"][1:])

    def timed(fn, steps):
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        n = sum(fn() for _ in range(steps))
        e1.record()
        torch.cuda.synchronize(dev)
        return n, e0.elapsed_time(e1)

    for _ in range(2):  # uncaptured, then captured
        batched()
        batched_streams()
    steps = max(1, min(args.steps, 3))
    leaves, ms = timed(batched, steps)
    s_leaves, s_ms = timed(batched_streams, steps)
    return {"metric": "prune leaves/s (circular-orbit tree)", "value": leaves / (ms * 1e-3),
            "unit": "leaves/s", "ms_per_step": ms / steps, "leaves_per_step": leaves // steps,
            "streams": {"value": s_leaves / (s_ms * 1e-3), "ms_per_step": s_ms / steps,
                        "note": (f"each run device-resident in its own CUDA graph, "
                                 f"{args.prune_streams} runs at once on their own streams")},
            "config": {"workload": "circ5_prune_circular_orbit_2^22",
                       "ref_segments": len(refs), "poly_order": 5,
                       "driver": "level-synchronous batch (loki_prune_run_batch, basis 2)"},
            "cpu_baseline": prune_cpu(circular=True) if not args.no_cpu_baseline else None}


def final_trials(cfg) -> int:
    return int(np.prod(cfg.get_param_grid_count(cfg.niters_ffa)))


def run_cpu_oracle(cfg, ts, nthreads: int = 0) -> tuple[float, int]:
    """One CPU search of the band sample with the oracle; returns (seconds, trials)."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    fold = O.ffa_execute(ts.ts_e, ts.ts_v, cfg, nthreads=nthreads)
    snr = O.boxcar_snr(O.fold_norm(fold[0]), cfg.score_widths, nthreads=nthreads)
    dt = time.perf_counter() - t0
    assert snr.shape[-1] == len(cfg.score_widths)
    return dt, final_trials(cfg)


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self

        def reader():
            for line in self.proc.stdout:
                self.rows.append([c.strip() for c in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=5)

    def summary(self) -> dict:
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def algorithmic_bytes(cfg, phase: str) -> float:
    """Algorithmic HBM bytes of one search phase (reads once + writes once)."""
    prof = 2 * cfg.nbins * 4
    n = cfg.niters_ffa

    def lvl(level):
        nseg = cfg.nsamps // (cfg.bseg_brute * 2**level)
        return nseg * int(np.prod(cfg.get_param_grid_count(level))) * prof

    if phase == "brutefold":
        return 2 * 4 * cfg.nsamps + lvl(0)
    if phase == "levels":  # levels 1..n-2 materialised (banded last two)
        return float(sum(lvl(level) + lvl(level - 1) for level in range(1, n - 1)))
    if phase == "final":  # read level n-2 once, write S/N of every final trial
        return float(lvl(n - 2) + final_trials(cfg) * len(cfg.score_widths) * 4)
    raise ValueError(phase)


def bench_gpu(args) -> dict | None:
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.replicas import max_over_ranks
    from pyloki_gb300.search import ffa_search
    from pyloki_gb300.timeseries import TimeSeries

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = make_cfg()
    ts_host = make_series(seed=1000 + rank)
    ts_e_pin = torch.from_numpy(ts_host.ts_e).pin_memory()
    ts_v_pin = torch.from_numpy(ts_host.ts_v).pin_memory()
    ts_dev = TimeSeries(ts_e_pin.to(dev), ts_v_pin.to(dev), cfg.tsamp)
    trials = final_trials(cfg)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    final_path = {}

    def one_step(events=None, storage="f32", norm=None):
        dyp = DynamicProgramming(ts_dev, cfg, device=dev, storage=storage)
        snr = dyp.search(band_bytes=args.band_bytes, phase_events=events, final=args.final,
                         norm=norm or args.norm)
        final_path["path"] = dyp.final_path
        return dyp, snr

    for _ in range(args.warmup):
        one_step()
    barrier()
    phases = {"brutefold": 0.0, "levels": 0.0, "final": 0.0}
    phase_launches = dict.fromkeys(phases, 0)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clocks:
        start.record()
        step_events = []
        for _ in range(args.steps):
            ev: list = []
            dyp, snr = one_step(ev)
            m = dyp.phase_marks
            phase_launches["brutefold"] += m["brutefold"] - m["start"]
            phase_launches["levels"] += m["levels"] - m["brutefold"]
            phase_launches["final"] += m["final"] - m["levels"]
            step_events.append(ev)
            del snr
        end.record()
        barrier()
    total_ms = start.elapsed_time(end)
    for ev in step_events:
        marks = dict(ev)
        phases["brutefold"] += marks["start"].elapsed_time(marks["brutefold"])
        phases["levels"] += marks["brutefold"].elapsed_time(marks["levels"])
        phases["final"] += marks["levels"].elapsed_time(marks["final"])
    total_ms = max_over_ranks(total_ms, dist, dev)  # the slowest replica
    ms_per_step = total_ms / args.steps

    # ---- end to end through the public API, host buffers ------------------
    ts_pinned = TimeSeries(ts_e_pin, ts_v_pin, cfg.tsamp)
    for _ in range(max(1, args.warmup // 2)):
        _, pg = ffa_search(ts_pinned, cfg, materialize=False, device=dev, norm=args.norm)
        pg.find_best_params(ignore_nan=True)
    barrier()
    t0 = time.perf_counter()
    best = None
    for _ in range(args.steps):
        _, pg = ffa_search(ts_pinned, cfg, materialize=False, device=dev, norm=args.norm)
        best = pg.find_best_params(ignore_nan=True)
        del pg
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, dist, dev)

    # the bit-exact normalisation, same search, for comparison (not the headline)
    norm_exact = None
    if args.norm == "fast":
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            _, snr = one_step(norm="exact")
            del snr
        e1.record()
        barrier()
        ex_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist, dev)
        norm_exact = {"value": world * trials / (ex_ms * 1e-3), "ms_per_step": ex_ms}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None

    dom = max(phases, key=phases.get)
    dom_ms = phases[dom] / args.steps
    ab = algorithmic_bytes(cfg, dom)
    peak, peak_kind = measured_peak_hbm()
    achieved = ab / (dom_ms * 1e-3) / 1e9
    dom_launches = max(1, phase_launches[dom] // args.steps)
    if dom == "final" and final_path["path"] == "tiled":
        dom_launches = 1  # the phase's other launches are its small table kernels
    traffic = None
    fpath = final_path["path"]
    if dom == "final" and fpath in FINAL_DRAM_BYTES_PER_TRIAL:
        # DRAM bytes per final trial from the ncu capture, x trials per launch
        traffic = FINAL_DRAM_BYTES_PER_TRIAL[fpath] * trials / dom_launches
    out = {
        "metric": METRIC,
        "value": world * trials / (ms_per_step * 1e-3),
        "unit": "trials/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded N(0,1) noise + 5 ms pulsar, accel 20 m/s^2, S/N 15)",
        "config": {"workload": WORKLOAD, "nsamps": cfg.nsamps, "tsamp": cfg.tsamp,
                   "nbins": cfg.nbins, "freq_hz": [50.0, 500.0], "accel_ms2": [-50.0, 50.0],
                   "widths": cfg.score_widths.tolist(), "levels": cfg.niters_ffa,
                   "final_grid": cfg.get_param_grid_count(cfg.niters_ffa).tolist(),
                   "trials_per_step": trials, "band_bytes": args.band_bytes,
                   "final_path": fpath,
                   "norm": ("rsqrt: S/N within 1e-5 of the bit-exact search"
                            if args.norm == "fast" else "exact: bit-identical S/N"),
                   "l2": "inputs larger than L2 (>51 GB read per step)",
                   "parallelism": f"replicas x{world}"},
        "phases_ms": {k: v / args.steps for k, v in phases.items()},
        "roofline": {"kernel": {"brutefold": "brutefold_seq_kernel (+phase_map_kernel)",
                                "levels": "ffa_level64_kernel (materialised levels)",
                                "final": FINAL_KERNEL[fpath]}[dom],
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "launches_per_step": dom_launches,
                     "algorithmic_bytes_per_launch": ab / dom_launches,
                     "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read+write per final trial at 2^21 "
                                       "samples x trials per launch"
                                       if traffic is not None else None},
        "e2e": {"value": world * trials / (e2e_ms * 1e-3), "unit": "trials/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": 2 * 4 * cfg.nsamps,
                "d2h_bytes_per_step": 8 + 4},
        "gpu_launches": sum(phase_launches.values()),
        "gpu_launches_per_step": {k: v // args.steps for k, v in phase_launches.items()},
        "clocks": clocks.summary(),
        "best_candidate": {k: float(v) for k, v in best.items()},
    }
    if norm_exact is not None:
        out["norm_exact"] = norm_exact
    if world == 1 and not args.no_cpu_baseline:
        cfg_b = cpu_band_cfg(args.cpu_band_hz)
        from oracle import oracle as O

        ts_b = make_series(seed=1000)
        dt, nt = run_cpu_oracle(cfg_b, ts_b)
        out["cpu_baseline"] = {"value": nt / dt, "unit": "trials/s",
                               "cores": O.max_threads(), "kind": "port",
                               "sample": f"same search restricted to "
                                         f"{500 - args.cpu_band_hz:g}-500 Hz ({nt} trials, "
                                         f"{dt:.1f} s)"}
    if not args.no_bf16:
        out["ffa_bf16"] = bench_bf16(args, dev, cfg, ts_dev, ts_host, one_step, trials,
                                     ms_per_step)
    if not args.no_batch:
        out["batch"] = bench_batch(args, dev)
    if not args.no_injections:
        out["injection"] = bench_injections(args, dev, peak)
    if not args.no_fourier:
        out["ffa_fourier"] = bench_fourier(args, dev)
    if world == 1:
        out["ffa_freq"] = bench_ffa_freq(args, dev)
    if not args.no_prune:
        out["prune"] = bench_prune_gpu(args, dev)
        if world == 1 and not args.no_cpu_baseline:
            out["prune"]["cpu_baseline"] = prune_cpu()
        if not args.no_fourier and world == 1:
            out["prune_fourier"] = bench_prune_fourier(args, dev)
        if world == 1:
            out["prune_circ"] = bench_prune_circ(args, dev)
        if not args.no_learned:
            out["prune"]["learned"] = bench_learned(args, dev)
        if not args.no_thresholds:
            from pyloki_gb300.branching import generate_branching_pattern

            out["threshold_design"] = bench_thresholds(
                args, dev, generate_branching_pattern(make_prune_cfg(), ref_seg=64))
    if dist is not None:
        dist.destroy_process_group()
    return out


INJ_NSAMPS = 2**21
FOURIER_NSAMPS = 2**20


def bench_fourier(args, dev) -> dict:
    """The Fourier-domain FFA (the reference's default, use_fourier=True) on
    the benchmark's acceleration grid at 2^20 samples, where every level can
    be materialised: complex brute fold, complex shift-add levels, irfft
    normalisation and boxcar S/N of every final trial. The time-domain search
    of the same grid is timed beside it."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.simulation import make_series as ms

    ts = ms(FOURIER_NSAMPS, 64e-6, freq=200.0, snr=15.0, ducy=0.05, accel=20.0, seed=1001)
    out = {"workload": "ffa_accel_search_2^20 (50-500 Hz, +-50 m/s^2, 64 bins)"}
    for name, fourier in (("fourier", True), ("time_domain", False)):
        cfg = make_cfg(nsamps=FOURIER_NSAMPS, use_fourier=fourier)
        dyp = DynamicProgramming(ts, cfg, device=dev)
        trials = int(np.prod(cfg.get_param_grid_count(cfg.niters_ffa)))

        def step():
            dyp.reset()
            return dyp.search(mode=1)

        for _ in range(max(args.warmup, 1)):
            step()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            snr = step()
        e1.record()
        torch.cuda.synchronize(dev)
        ms_step = e0.elapsed_time(e1) / args.steps
        best = float(torch.nan_to_num(snr, nan=float("-inf")).max())
        marks: list = []
        dyp.reset()
        dyp.search(mode=1, phase_events=marks)
        torch.cuda.synchronize(dev)
        phases = {marks[i][0]: marks[i - 1][1].elapsed_time(marks[i][1])
                  for i in range(1, len(marks))}
        out[name] = {"trials_per_s": trials / (ms_step * 1e-3), "ms_per_step": ms_step,
                     "trials": trials, "best_snr": best, "phases_ms": phases}
    return out


def bench_ffa_freq(args, dev) -> dict:
    """The plain FFA frequency search that the reference can run on a CPU:
    one series of 2^20 samples at 64 us with a von Mises pulse (5 % duty,
    P = 0.5 s, folded S/N 12 by the reference's calibration), periods
    0.1-1 s, 64 bins, widths 1-32. The GPU search and the CPU oracle (all
    host threads) of the whole search; the best candidate of each."""
    import torch

    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.pulse import PulseSignalConfig
    from pyloki_gb300.timeseries import TimeSeries

    cfg = PulsarSearchConfig(nsamps=2**20, tsamp=64e-6, nbins=64, eta=1.0,
                             param_limits=ParamLimits.from_taylor((1.0, 10.0)).limits,
                             ducy_max=0.5, wtsp=2.0, use_fourier=False)
    sig = PulseSignalConfig(period=0.5, dt=64e-6, nsamps=2**20, snr=12.0, ducy=0.05)
    ts = sig.generate(shape="von_mises", seed=1100, device=dev)
    trials = final_trials(cfg)
    dyp = DynamicProgramming(ts, cfg, device=dev)

    def step():
        dyp.reset()
        return dyp.search(norm=args.norm)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        snr = step()
    e1.record()
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / args.steps
    best = snr.reshape(-1, snr.shape[-1]).amax(dim=1)
    i = int(torch.argmax(best))
    f = cfg.get_param_arr(cfg.get_dparams(cfg.niters_ffa))[-1]
    out = {"workload": "ffa_freq_search_2^20 (periods 0.1-1 s, 64 bins, widths 1-32)",
           "value": trials / (ms * 1e-3), "unit": "trials/s", "ms_per_step": ms,
           "trials": trials, "final_path": dyp.final_path,
           "best": {"snr": float(best[i]), "period_s": float(1 / f[i])}}
    if not args.no_cpu_baseline:
        from oracle import oracle as O

        host = TimeSeries(ts.ts_e.cpu().numpy(), ts.ts_v.cpu().numpy(), cfg.tsamp)
        dt, nt = run_cpu_oracle(cfg, host)
        out["cpu_baseline"] = {"value": nt / dt, "unit": "trials/s", "cores": O.max_threads(),
                               "kind": "port", "sample": f"the whole search ({nt} trials)",
                               "seconds": dt}
    return out


def injection_cfgs(n: int, seed: int = 4000):
    """Seeded injection set: periods 2-50 ms, S/N 8-30, duty cycles 0.02-0.3,
    accelerations +-50 m/s^2 and jerks +-0.1 m/s^3 (Taylor modulation), 2^21
    samples of 64 us; shapes and pulse phases per injection."""
    from pyloki_gb300.pulse import PulseSignalConfig

    rng = np.random.default_rng(seed)
    cfgs = [PulseSignalConfig(period=float(p), dt=64e-6, nsamps=INJ_NSAMPS, snr=float(s),
                              ducy=float(d), mod_kwargs={"acc": float(a), "jerk": float(j)})
            for p, s, d, a, j in zip(rng.uniform(2e-3, 5e-2, n), rng.uniform(8, 30, n),
                                     rng.uniform(0.02, 0.3, n), rng.uniform(-50, 50, n),
                                     rng.uniform(-0.1, 0.1, n))]
    shapes = [("gaussian", "von_mises", "boxcar")[i % 3] for i in range(n)]
    return cfgs, shapes, rng.uniform(0, 1, n)


def bench_injections(args, dev, peak: float) -> dict:
    """Synthetic injection set on the device (PulseSignalConfig.generate for
    every injection): proper time, template, noise and calibration folds in
    one pass (which also stores noise and template in the output arrays), the
    calibration, and the in-place scaling to the float32 series, kept in HBM. Device time per
    kernel phase from CUDA events; wall time of the public call (host
    preparation of the CDF tables included). CPU baseline: the numpy port on
    two injections of the same set."""
    import torch

    from oracle import pulse_oracle as PO
    from pyloki_gb300 import _lib
    from pyloki_gb300.pulse import _Batch, generate_injections

    n = args.injections
    cfgs, shapes, phis = injection_cfgs(n)
    ts_e = torch.empty((n, INJ_NSAMPS), dtype=torch.float32, device=dev)
    ts_v = torch.empty_like(ts_e)
    generate_injections(cfgs[:8], shapes[:8], phis[:8], seed=1, device=dev)  # warm-up
    stream = torch.cuda.current_stream(dev)
    times = {}
    for rep in range(2):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        batch = _Batch(cfgs, shapes, phis, 1, dev)
        t_prep = time.perf_counter() - t0
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        before = _lib.load().loki_launch_count()
        ev[0].record(stream)
        folds = batch.fold(None, keep=(ts_e, ts_v))
        ev[1].record(stream)
        scales = batch.calibrate(folds, 5, 1e-2)
        ev[2].record(stream)
        batch.apply(scales, ts_e, ts_v)
        ev[3].record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        launches = _lib.load().loki_launch_count() - before
        times = {"fold_ms": ev[0].elapsed_time(ev[1]), "calibrate_ms": ev[1].elapsed_time(ev[2]),
                 "apply_ms": ev[2].elapsed_time(ev[3]), "device_ms": ev[0].elapsed_time(ev[3]),
                 "host_prep_ms": t_prep * 1e3, "wall_ms": wall * 1e3, "launches": launches}
    samples = n * INJ_NSAMPS
    meas = scales[:, 3].cpu().numpy()
    # apply: noise and template read, ts_e and ts_v written, 4 bytes each
    apply_bytes = 16 * samples
    apply_gbs = apply_bytes / (times["apply_ms"] * 1e-3) / 1e9
    # CPU: the numpy port of generate() on two injections of the set
    rng = np.random.default_rng(9)
    t0 = time.perf_counter()
    for i in range(2):
        c = cfgs[i]
        noise = rng.standard_normal(INJ_NSAMPS, dtype=np.float32)
        PO.generate(c.period, c.dt, c.nsamps, c.snr, c.ducy, noise, shape=shapes[i],
                    phi0=float(phis[i]), kind="derivative", params=c.mod_kwargs,
                    exact_folds=True)
    cpu_per = (time.perf_counter() - t0) / 2
    return {"metric": "injections/s", "value": n / (times["wall_ms"] * 1e-3),
            "unit": "injections/s", "device_injections_per_s": n / (times["device_ms"] * 1e-3),
            "samples_per_s_device": samples / (times["device_ms"] * 1e-3),
            "injections": n, "nsamps": INJ_NSAMPS, **times,
            "calibrated_snr_abs_err_median": float(np.median(np.abs(
                meas - np.array([c.snr for c in cfgs])))),
            "roofline_apply": {"bound": "hbm", "achieved": apply_gbs, "peak": peak,
                               "unit": "GB/s", "frac": apply_gbs / peak,
                               "algorithmic_bytes": apply_bytes},
            "fold_samples_per_s": samples / (times["fold_ms"] * 1e-3),
            "cpu_baseline": {"value": 1.0 / cpu_per, "unit": "injections/s", "cores": 1,
                             "kind": "port",
                             "sample": "numpy port of generate() on 2 injections of the set"},
            "workload": f"{n} injections x 2^21 samples (Taylor modulation, three shapes)"}


def bench_thresholds(args, dev, branching_pattern) -> dict:
    """Dynamic threshold-scheme design for the pruning workload's branching
    pattern, with the design parameters of the reference's threshold notebook:
    100 thresholds, 30 probability bins, 1024 trials per fold set, S/N 10,
    beam 2.5, improved mode, 11 neighbours."""
    import torch

    from pyloki_gb300.thresholds import DynamicThresholdScheme

    bp = np.asarray(branching_pattern, np.float64)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ds = DynamicThresholdScheme(bp, 0.1, 64, ntrials=1024, nprobs=30, prob_min=0.05,
                                snr_final=10.0, nthresholds=100, ducy_max=0.3, wtsp=1.5,
                                beam_width=2.5, mode="improved", seed=1, device=dev)
    ds.run(thres_neigh=11)
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    path = ds.best_path()
    return {"metric": "threshold design seconds", "value": dt, "unit": "s",
            "higher_is_better": False, "stages": len(bp), "nthresholds": 100, "nprobs": 30,
            "ntrials": 1024, "mode": "improved", "simulate_launches": ds.sim.launches,
            "final_states": int((~ds.states[-1]["is_empty"]).sum()),
            "best_path_stages": len(path),
            "note": "the reference's notebook reports 121.5 s for a 127-stage design with "
                    "these parameters on its CPU (numba)"}


class PruneInjections:
    """Series of the pruning workload made on the GPU by the reference's
    generator (``pulse.PulseSignalConfig``: folded S/N calibrated on the
    folds, ``simulation/pulse.py:71-118``): a 3 ms pulsar (von Mises, 5 %
    duty, S/N 10) in a circular orbit with P_orb 2-10 h, x 0.1-2 lt-s and an
    orbital phase drawn from the seed; or the same noise alone. 2^22 samples
    of 64 us, made ``batch`` seeds at a time."""

    def __init__(self, dev, batch: int = 32) -> None:
        self.dev = dev
        self.batch = batch
        self._cache: dict = {}

    @staticmethod
    def signal(seed: int):
        from pyloki_gb300.pulse import PulseSignalConfig

        rng = np.random.default_rng(seed)
        orb = {"p_orb": rng.uniform(2.0, 10.0) * 3600.0, "x_orb": rng.uniform(0.1, 2.0),
               "psi": rng.uniform(0.0, 2 * np.pi)}
        return PulseSignalConfig(period=3e-3, dt=64e-6, nsamps=2**22, snr=10.0, ducy=0.05,
                                 mod_type="circular", mod_kwargs=orb)

    def __call__(self, seed: int, inject: bool):
        from pyloki_gb300.pulse import generate_injections
        from pyloki_gb300.timeseries import TimeSeries

        if not inject:
            return self.signal(seed).generate_noise(seed=seed, device=self.dev)
        base = seed - seed % self.batch
        hit = self._cache.get("inj")
        if hit is None or hit[0] != base:
            cfgs = [self.signal(s) for s in range(base, base + self.batch)]
            b = generate_injections(cfgs, shape="von_mises", seed=base, device=self.dev)
            hit = self._cache["inj"] = (base, b)
        b = hit[1]
        i = seed - base
        return TimeSeries(b.ts_e[i], b.ts_v[i], b.dt)


def clopper_pearson(k: int, n: int, conf: float = 0.95) -> tuple[float, float]:
    """Exact binomial confidence interval of k successes in n trials."""
    from scipy import stats

    a = (1 - conf) / 2
    lo = 0.0 if k == 0 else float(stats.beta.ppf(a, k, n - k + 1))
    hi = 1.0 if k == n else float(stats.beta.ppf(1 - a, k + 1, n - k))
    return lo, hi


def bench_learned(args, dev) -> dict:
    """Learned branch proposal on the pruning workload: the MLP is trained on
    the GPU on branch statistics of plain runs over seeded injections, then
    plain and learned pruning run on held-out injections and noise-only
    series. The full design is 10,000 / 1,000 / 1,000 series; the default run
    takes a bounded sample (--learned-train / --learned-test)."""
    from pyloki_gb300.learned import study

    cfg = make_prune_cfg()
    nseg = cfg.nsamps // cfg.bseg_ffa
    n_tr, n_te = args.learned_train, args.learned_test
    gen = PruneInjections(dev)
    res = study(cfg, prune_thresholds(nseg), gen,
                train_seeds=list(range(10_000, 10_000 + n_tr)),
                test_seeds=list(range(20_000, 20_000 + n_te)),
                noise_seeds=list(range(30_000, 30_000 + n_te)),
                budget=args.learned_budget, lookahead=16, per_level=2048, epochs=6,
                score_share=args.learned_score_share,
                max_sugg=PRUNE_MAX_SUGG, batch_size=PRUNE_BATCH, device=dev)
    inj, noise = res["injected"], res["noise"]
    for bud, row in res["budgets"].items():
        k = sum(r["learned"][int(bud)]["best"] >= r["plain_best"] - 1e-3 for r in inj)
        row["recall_ci95"] = clopper_pearson(int(k), len(inj)) if inj else None
        fa = sum(r["learned"][int(bud)]["best"] >= res["det_snr"] for r in noise)
        row["false_alarm_ci95"] = clopper_pearson(int(fa), len(noise)) if noise else None
    det = sum(r["plain_best"] >= res["det_snr"] for r in inj)
    res["plain_detection"] = {"rate": det / max(len(inj), 1),
                              "ci95": clopper_pearson(int(det), len(inj)) if inj else None}
    res["workload"] = PRUNE_WORKLOAD
    res["sample"] = (f"{n_tr} training injections, {n_te} held-out injections, {n_te} "
                     "noise-only series (seeded; GPU generator with the reference's S/N "
                     "calibration)")
    if len(inj) >= 100:  # per-series records stay in the detail file only for small studies
        res.pop("injected")
        res.pop("noise")
    return res


def batch_cfg(n: int):
    """Jerk search of one batch series of n = 2^k samples: f 50-500 Hz,
    accel +-30 m/s^2, jerk +-0.05 m/s^3, 64 bins, widths 1-16."""
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig

    return PulsarSearchConfig(
        nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
        param_limits=ParamLimits.from_taylor((50.0, 500.0), accel=(-30.0, 30.0),
                                             jerk=(-0.05, 0.05)).limits,
        ducy_max=0.25, wtsp=2.0, use_fourier=False, bseg_brute=16384)


def make_batch_series(n_series: int, seed: int = 3000):
    """Seeded batch: lengths uniform in [2^20, 2^23]; one series in ten carries
    a pulsar (P 2-20 ms, accel +-30, jerk +-0.05, S/N 8-20)."""
    from pyloki_gb300.batch import cfg3_lengths
    from pyloki_gb300.simulation import make_series as ms

    lengths = cfg3_lengths(256, seed)[:n_series]
    rng = np.random.default_rng(seed + 1)
    out, injected = [], []
    for i, n in enumerate(lengths):
        if rng.random() < 0.1:
            p = rng.uniform(2e-3, 20e-3)
            out.append(ms(int(n), 64e-6, freq=1.0 / p, snr=rng.uniform(8.0, 20.0), ducy=0.05,
                          accel=rng.uniform(-30.0, 30.0), jerk=rng.uniform(-0.05, 0.05),
                          seed=seed + 10 + i))
            injected.append(i)
        else:
            out.append(ms(int(n), 64e-6, seed=seed + 10 + i))
    return out, injected


def bench_batch(args, dev) -> dict:
    """Batched pattern on a bounded sample of the 256-series batch: the plain
    path (one FP32 search per series, eager launches) against the batched
    path (segment-stacked chunks, CUDA-graph replay, tuned chunk and band
    sizes) with FP32 storage, and with bfloat16 storage plus FP64 re-scoring
    of the kept candidates; recall is the batched-bf16 recovery of the plain
    path's best S/N per series (FP64 S/N within 1e-3)."""
    import torch

    from pyloki_gb300.batch import BatchedSearch, Tuner, sequential_search

    from pyloki_gb300.timeseries import TimeSeries

    host, injected = make_batch_series(args.batch_series)
    # pinned host buffers: the copies are part of every pass
    series = [TimeSeries(torch.from_numpy(ts.ts_e).pin_memory(),
                         torch.from_numpy(ts.ts_v).pin_memory(), ts.tsamp) for ts in host]

    def timed(fn) -> tuple[float, object]:
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t0) * 1e3, out

    ms_plain, plain = timed(lambda: sequential_search(series, batch_cfg, device=dev, k=BATCH_K))
    ms_plain, plain = timed(lambda: sequential_search(series, batch_cfg, device=dev, k=BATCH_K))
    tuner = Tuner()
    res = {}
    for name, storage, rescore in (("batched_f32", "f32", False),
                                   ("batched_bf16_rescored", "bf16", True)):
        bs = BatchedSearch(series, batch_cfg, device=dev, k=BATCH_K, storage=storage,
                           rescore=rescore, tuner=tuner)
        t0 = time.perf_counter()
        bs.prepare()
        prep_s = time.perf_counter() - t0
        bs.run()  # warm replay
        ms_b, cands = timed(bs.run)
        res[name] = {"ms": ms_b, "trials_per_s": bs.trials() / (ms_b * 1e-3),
                     "speedup_vs_plain": ms_plain / ms_b, "prepare_s": prep_s,
                     "graph_launches": bs.graph_launches, "kernel_launches": bs.launches,
                     "plan": {str(n): {"chunk": p.chunk, "band_bytes": p.band_bytes}
                              for n, p in bs.plan.items()},
                     "_cands": cands}
    trials = bs.trials()
    bf = res["batched_bf16_rescored"].pop("_cands")
    f32 = res["batched_f32"].pop("_cands")
    same_f32 = all(np.array_equal(a.snr_search, b.snr_search) for a, b in zip(f32, plain))
    rec = [bool(b.snr[0] >= p.snr[0] - 1e-3) for b, p in zip(bf, plain)]
    rec_inj = [rec[i] for i in injected]
    lengths = {}
    for ts in series:
        n = 1 << (len(ts.ts_e).bit_length() - 1)
        lengths[str(n)] = lengths.get(str(n), 0) + 1
    return {"metric": "period-trials/s (batch)", "workload": BATCH_WORKLOAD,
            "series": len(series), "series_per_length": lengths, "trials_per_pass": trials,
            "k": BATCH_K, "plain_ms": ms_plain,
            "plain_trials_per_s": trials / (ms_plain * 1e-3), **res,
            "batched_f32_equals_plain_topk": same_f32,
            "recall_vs_plain": float(np.mean(rec)),
            "recall_vs_plain_injected": float(np.mean(rec_inj)) if rec_inj else None,
            "injected_series": len(injected),
            "note": "pinned host series, H2D copies inside every pass; lengths truncated "
                    "to powers of two; bf16 candidates re-scored in FP64 from the samples"}


def bench_bf16(args, dev, cfg, ts_dev, ts_host, one_step, trials, f32_ms) -> dict:
    """The same search with bfloat16 fold storage (FP32 arithmetic): device
    throughput, then the S/N error against the FP64 oracle on the top
    candidates plus a random sample of trials, and the FP64 GPU re-scoring of
    the same trials against the same oracle."""
    import torch

    from oracle import oracle as O

    for _ in range(args.warmup):
        one_step(storage="bf16")
    torch.cuda.synchronize(dev)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    phases = {"brutefold": 0.0, "levels": 0.0, "final": 0.0}
    step_events = []
    start.record()
    for _ in range(args.steps):
        ev: list = []
        dyp, snr = one_step(ev, storage="bf16")
        step_events.append(ev)
        del snr
    end.record()
    torch.cuda.synchronize(dev)
    ms = start.elapsed_time(end) / args.steps
    for ev in step_events:
        marks = dict(ev)
        phases["brutefold"] += marks["start"].elapsed_time(marks["brutefold"]) / args.steps
        phases["levels"] += marks["brutefold"].elapsed_time(marks["levels"]) / args.steps
        phases["final"] += marks["levels"].elapsed_time(marks["final"]) / args.steps
    # precision: top candidates + random trials against the FP64 oracle
    dyp, snr = one_step(storage="bf16")
    flat = snr.reshape(-1, snr.shape[-1])
    # trials with an empty bin (v = 0) have S/N NaN, as in the reference
    best = torch.nan_to_num(flat.amax(dim=1), nan=float("-inf"))
    top = torch.topk(best, BF16_TOP).indices.cpu().numpy()
    rng = np.random.default_rng(7)
    pick = np.unique(np.r_[top, rng.integers(0, flat.shape[0], BF16_SAMPLE)])
    t0 = time.perf_counter()
    ref = O.boxcar_snr_f64(O.ffa_trials(ts_host.ts_e, ts_host.ts_v, cfg, pick, f64=True),
                           cfg.score_widths)
    t_oracle = time.perf_counter() - t0
    got = flat[torch.from_numpy(pick).to(dev)].double().cpu().numpy()
    cand = torch.from_numpy(top).to(dev)
    torch.cuda.synchronize(dev)
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    r0.record()
    resc_top = dyp.rescore(cand)
    r1.record()
    torch.cuda.synchronize(dev)
    resc = dyp.rescore(torch.from_numpy(pick).to(dev)).cpu().numpy()
    fin = np.isfinite(ref) & np.isfinite(got)
    nan_mismatch = int((np.isnan(ref) != np.isnan(got)).sum())
    err = np.where(fin, np.abs(got - ref), 0.0)
    rel = err / np.maximum(np.abs(np.where(fin, ref, 1.0)), 1.0)
    rfin = np.isfinite(ref) & np.isfinite(resc)
    rerr = np.where(rfin, np.abs(resc - ref), 0.0) / np.maximum(
        np.abs(np.where(rfin, ref, 1.0)), 1.0)
    in_top = np.isin(pick, top)
    del resc_top
    return {
        "value": trials / (ms * 1e-3), "unit": "trials/s", "ms_per_step": ms,
        "speedup_vs_f32_storage": f32_ms / ms, "dtype": "bf16 storage, f32 arithmetic",
        "phases_ms": phases,
        "snr_error_vs_fp64": {
            "trials": int(len(pick)), "top_candidates": BF16_TOP,
            "max_abs": float(err.max()), "max_rel": float(rel.max()),
            "median_abs": float(np.median(err[fin])),
            "nan_mismatch": nan_mismatch,
            "top_max_abs": float(err[in_top].max()),
            "rescored_max_rel": float(rerr.max()),
            "rescore_ms_top": r0.elapsed_time(r1),
            "oracle_s": t_oracle,
            "note": "rel = |err| / max(|S/N_fp64|, 1); rescored = FP64 GPU re-scoring "
                    "from the FP32 level-0 fold"},
    }


def bench_reference(args) -> dict | None:
    """CPU oracle (all host threads) on a bounded band of the same search."""
    if int(os.environ.get("RANK", "0")) != 0:
        return None
    from oracle import oracle as O

    cfg_b = cpu_band_cfg(args.cpu_band_hz)
    ts_b = make_series(seed=1000)
    for _ in range(args.warmup):
        run_cpu_oracle(cfg_b, ts_b)
    times = []
    nt = final_trials(cfg_b)
    for _ in range(args.steps):
        dt, nt = run_cpu_oracle(cfg_b, ts_b)
        times.append(dt)
    value = nt / (sum(times) / len(times))
    out = {
        "metric": METRIC, "value": value, "unit": "trials/s", "impl": "reference",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "sample_band_hz": [500 - args.cpu_band_hz, 500.0],
                   "trials_per_step": nt},
        "cpu_baseline": {"value": value, "unit": "trials/s", "cores": O.max_threads(),
                         "kind": "port",
                         "sample": f"{500 - args.cpu_band_hz:g}-500 Hz band of the search "
                                   f"({nt} trials per step)"},
        "e2e": {"value": value, "unit": "trials/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if not args.no_prune:
        p = prune_cpu()
        out["prune"] = {"metric": "prune leaves/s", "value": p["value"], "unit": "leaves/s",
                        "config": {"workload": PRUNE_WORKLOAD}, "cpu_baseline": p,
                        "e2e": {"value": p["value"], "unit": "leaves/s",
                                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out


def profile_once(args) -> None:
    """One search of the benchmark workload (optionally on a shorter series)
    with no timing; the command that the ncu summaries are captured from."""
    import torch

    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.simulation import make_series as ms

    n = 2**args.nsamps_log2
    cfg = PulsarSearchConfig(
        nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
        param_limits=ParamLimits.from_taylor((50.0, 500.0), accel=(-50.0, 50.0)).limits,
        ducy_max=0.25, wtsp=2.0, use_fourier=False,
        bseg_brute=16384 if n == 2**23 else 0)
    ts = ms(n, 64e-6, freq=200.0, snr=15.0, ducy=0.05, accel=20.0, seed=1000)
    dyp = DynamicProgramming(ts, cfg, device=torch.device("cuda", 0))
    snr = dyp.search(band_bytes=args.band_bytes, final=args.final, norm=args.norm)
    torch.cuda.synchronize()
    print(json.dumps({"profile_once": True, "nsamps": n, "levels": cfg.niters_ffa,
                      "final_grid": cfg.get_param_grid_count(cfg.niters_ffa).tolist(),
                      "launches": dyp.launches, "snr_shape": list(snr.shape)}))


def profile_fourier_once(args) -> None:
    """One Fourier-domain search of the benchmark grid at 2^20 samples after a
    warm-up, with no timing; the command the Fourier ncu summaries use."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.simulation import make_series as ms

    cfg = make_cfg(nsamps=FOURIER_NSAMPS, use_fourier=True)
    ts = ms(FOURIER_NSAMPS, 64e-6, freq=200.0, snr=15.0, ducy=0.05, accel=20.0, seed=1001)
    dyp = DynamicProgramming(ts, cfg, device=torch.device("cuda", 0))
    for _ in range(2):
        dyp.reset()
        snr = dyp.search(mode=1)
    torch.cuda.synchronize()
    print(json.dumps({"profile_fourier_once": True, "nsamps": FOURIER_NSAMPS,
                      "best_snr": float(torch.nan_to_num(snr, nan=-1.0).max())}))


def profile_inject_once(args) -> None:
    """One injection set of 64 x 2^21 samples after a warm-up, with no timing;
    the command the generator's ncu summaries are captured from."""
    import torch

    from pyloki_gb300.pulse import generate_injections

    dev = torch.device("cuda", 0)
    cfgs, shapes, phis = injection_cfgs(64)
    generate_injections(cfgs[:4], shapes[:4], phis[:4], seed=1, device=dev)
    b = generate_injections(cfgs, shapes, phis, seed=1, device=dev)
    torch.cuda.synchronize(dev)
    print(json.dumps({"profile_inject_once": True, "injections": len(cfgs),
                      "nsamps": INJ_NSAMPS,
                      "median_snr_err": float(np.median(np.abs(
                          b.scales[:, 3].cpu().numpy() - [c.snr for c in cfgs])))}))


def profile_prune_once(args) -> None:
    """One pruning run of the pruning workload after one warm-up run, with no
    timing; the command the pruning ncu summaries are captured from."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning

    dev = torch.device("cuda", 0)
    cfg = make_prune_cfg()
    ts, _ = make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=dev)
    dyp.initialize()
    dyp.execute()
    nseg = dyp.nsegments
    prn = Pruning(dyp, prune_thresholds(nseg), max_sugg=PRUNE_MAX_SUGG, batch_size=PRUNE_BATCH)
    for _ in range(2):
        res = prn.execute(nseg // 2)
    torch.cuda.synchronize()
    print(json.dumps({"profile_prune_once": True, "levels": nseg - 1,
                      "leaves": sum(st.n_leaves for st in res["level_stats"][1:]),
                      "launches_per_run": prn.launches // 2}))


def profile_prune_batch_once(args) -> None:
    """One batched pruning step (``PruneBlockBatch``, the first call of a
    fresh runner, so its kernels are launched directly) over args.prune_runs
    reference segments, with no timing; the command the batched-pruning ncu
    summaries are captured from. ``--prune-circ``: the circular-orbit tree
    of order 5 on the same series."""
    import torch

    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBlockBatch

    dev = torch.device("cuda", 0)
    cfg = make_prune_cfg(circular=args.prune_circ)
    ts, _ = make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=dev)
    dyp.initialize()
    dyp.execute()
    nseg = dyp.nsegments
    refs = [int(r) for r in np.linspace(4, nseg - 5, args.prune_runs).round()]
    res = PruneBlockBatch(prune_thresholds(nseg), max_sugg=PRUNE_MAX_SUGG,
                          batch_size=PRUNE_BATCH).run([(dyp, r) for r in refs])
    torch.cuda.synchronize()
    print(json.dumps({"profile_prune_batch_once": True, "runs": len(refs),
                      "leaves": sum(st.n_leaves for r in res for st in r["level_stats"][1:])}))


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--band-bytes", type=int, default=1 << 30)
    ap.add_argument("--final", choices=["auto", "tiled", "banded", "level"], default="auto",
                    help="how the last two FFA levels run")
    ap.add_argument("--norm", choices=["exact", "fast"], default="fast",
                    help="profile normalisation of the tiled final levels: fast = e * rsqrt(v) "
                         "(S/N within 1e-5 of exact), exact = bit-identical to the reference")
    ap.add_argument("--cpu-band-hz", type=float, default=4.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-bf16", action="store_true",
                    help="skip the bfloat16-storage search and its FP64 error check")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched multi-series measurement")
    ap.add_argument("--batch-series", type=int, default=BATCH_SERIES,
                    help="series of the seeded 256-series batch to search")
    ap.add_argument("--profile-fourier-once", action="store_true",
                    help="two untimed Fourier-domain searches at 2^20 (the Fourier ncu command)")
    ap.add_argument("--profile-inject-once", action="store_true",
                    help="one untimed 64-injection set (the generator ncu command)")
    ap.add_argument("--prune-workers", type=int, default=PRUNE_WORKERS,
                    help="host threads (each with its own stream) of the multi-run pruning")
    ap.add_argument("--prune-streams", type=int, default=PRUNE_STREAMS,
                    help="concurrent device-resident runs of the batched pruning measurement")
    ap.add_argument("--prune-runs", type=int, default=PRUNE_MULTI_RUNS,
                    help="reference segments of the multi-run pruning")
    ap.add_argument("--no-fourier", action="store_true",
                    help="skip the Fourier-domain FFA section")
    ap.add_argument("--no-injections", action="store_true",
                    help="skip the synthetic injection-set section")
    ap.add_argument("--injections", type=int, default=1024,
                    help="injections of 2^21 samples in the injection-set section")
    ap.add_argument("--no-thresholds", action="store_true",
                    help="skip the threshold-scheme design measurement")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned branch proposal study")
    ap.add_argument("--learned-train", type=int, default=16)
    ap.add_argument("--learned-test", type=int, default=16)
    ap.add_argument("--learned-score-share", type=float, default=0.5,
                    help="share of each level's parent budget given to the best-scoring "
                         "parents (the rest is ranked by the network)")
    ap.add_argument("--learned-budget", type=int, nargs="+", default=[4096, 8192, 16384],
                    help="parents expanded per level under the learned proposal")
    ap.add_argument("--no-prune", action="store_true",
                    help="skip the enumerate-prune (leaves/s) measurement")
    ap.add_argument("--profile-once", action="store_true",
                    help="run exactly one search (for ncu captures) and exit")
    ap.add_argument("--profile-prune-once", action="store_true",
                    help="run the pruning workload twice (warm-up + one run) and exit")
    ap.add_argument("--prune-circ", action="store_true",
                    help="with --profile-prune-batch-once: the circular-orbit tree of order 5")
    ap.add_argument("--profile-prune-batch-once", action="store_true",
                    help="one batched pruning step over --prune-runs segments, then exit")
    ap.add_argument("--detail-out", default=None,
                    help="also write the full result (every side study) to this JSON file")
    ap.add_argument("--nsamps-log2", type=int, default=23,
                    help="series length for --profile-once (smaller ncu cases)")
    args = ap.parse_args()
    if args.profile_once:
        profile_once(args)
        return
    if args.profile_prune_once:
        profile_prune_once(args)
        return
    if args.profile_prune_batch_once:
        profile_prune_batch_once(args)
        return
    if args.profile_inject_once:
        profile_inject_once(args)
        return
    if args.profile_fourier_once:
        profile_fourier_once(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    out = bench_reference(args) if args.impl == "reference" else bench_gpu(args)
    if out is None:
        return
    if args.detail_out:
        Path(args.detail_out).parent.mkdir(parents=True, exist_ok=True)
        Path(args.detail_out).write_text(json.dumps(out, indent=1))
    # one line per side study first, the compact headline last
    for key in SECTIONS:
        if key in out:
            print(json.dumps({"section": key, **_compact_section(out[key])}), flush=True)
    if isinstance(out.get("prune"), dict):
        for key in ("multi_run", "learned"):
            if isinstance(out["prune"].get(key), dict):
                print(json.dumps({"section": f"prune.{key}",
                                  **_compact_section(out["prune"][key])}), flush=True)
    print(json.dumps(headline(out)), flush=True)


# side studies printed on their own lines before the headline
SECTIONS = ("ffa_bf16", "ffa_precision", "batch", "injection", "ffa_fourier", "prune_fourier",
            "prune_circ", "threshold_design")
HEADLINE_KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                 "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "impl",
                 "gpu_launches", "clocks")


def _round(x):
    if isinstance(x, float):
        return float(f"{x:.6g}")
    if isinstance(x, dict):
        return {k: _round(v) for k, v in x.items()}
    if isinstance(x, list):
        return [_round(v) for v in x]
    return x


def _compact_section(sec: dict) -> dict:
    """A side study without its long per-item lists (kept in the detail file)."""
    return _round({k: v for k, v in sec.items()
                   if not (isinstance(v, list) and len(v) > 8)})


def headline(out: dict) -> dict:
    """The last stdout line: the period-trials/s headline with its roofline,
    CPU baseline and end-to-end figures, and the prune leaves/s headline as a
    small sub-object; a few hundred bytes to about 2 KB."""
    h = {k: out[k] for k in HEADLINE_KEYS if k in out}
    cfg = out.get("config", {})
    h["config"] = {k: cfg[k] for k in ("workload", "nsamps", "trials_per_step", "final_grid",
                                       "widths", "norm", "l2", "parallelism", "sample_band_hz")
                   if k in cfg}
    if "norm_exact" in out:
        h["norm_exact"] = out["norm_exact"]
    for k in ("roofline", "cpu_baseline", "e2e"):
        if k in out:
            h[k] = {kk: vv for kk, vv in out[k].items()
                    if kk not in ("traffic_source", "sample", "peak_kind",
                                  "algorithmic_bytes_per_launch") or k == "cpu_baseline"}
    if "roofline" in h:  # the kernel's name only; the detail file has the description
        h["roofline"]["kernel"] = h["roofline"]["kernel"].split(" (")[0]
    if "prune" in out:
        p = out["prune"]
        sub = {k: p[k] for k in ("metric", "value", "unit", "ms_per_step", "leaves_per_step",
                                 "speedup_vs_plain") if k in p}
        if "plain" in p:
            sub["plain"] = {"value": p["plain"]["value"], "ms_per_run": p["plain"]["ms_per_run"]}
        pc = p.get("config", {})
        sub["config"] = {k: pc[k] for k in ("workload", "thresholds", "ref_segments", "driver")
                         if k in pc}
        if "streams" in p:
            sub["streams"] = {"value": p["streams"]["value"],
                              "ms_per_step": p["streams"]["ms_per_step"]}
        for k in ("roofline", "cpu_baseline", "e2e"):
            if k in p:
                sub[k] = {kk: vv for kk, vv in p[k].items()
                          if kk in ("kernel", "bound", "achieved", "peak", "unit", "frac",
                                    "traffic", "value", "cores", "kind", "ms_per_step",
                                    "h2d_bytes_per_step", "d2h_bytes_per_step")}
        if "roofline" in sub:
            sub["roofline"]["kernel"] = sub["roofline"]["kernel"].split(" (")[0]
        if "learned" in p and isinstance(p["learned"], dict):
            lh = p["learned"].get("headline")
            if lh:
                sub["learned"] = lh
        h["prune"] = sub
    return _round(h)


if __name__ == "__main__":
    main()

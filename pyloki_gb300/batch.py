"""Many series in one pass: batched FFA search with CUDA graphs and a tuner.

The reference searches one series per call (``search.py:17-53``) and spreads
runs over worker processes. Here series of equal (power-of-two) length are
concatenated and searched together: their segments are stacked along the
segment axis, so each DP level, the banded final levels and the fused scoring
run once for the whole chunk of series (``DynamicProgramming(nbatch=...)``).
Every chunk's whole search (brute fold, levels, final bands, NaN-safe top-k)
is captured once in a CUDA graph and replayed for the next chunk of the same
shape, so a chunk costs one graph launch and no host round trips.

The chunk size (series per pass) and the band size of the final levels are
chosen per shape by ``Tuner``, which times the candidates on the device and
keeps the fastest (optionally persisted as JSON).

Series of uneven length are first truncated to the largest power of two that
fits (``pow2_length``); each length forms a group with its own grids.
"""

from __future__ import annotations

import json
import os
from collections.abc import Callable, Sequence
from dataclasses import dataclass, field

import numpy as np
import torch

from pyloki_gb300 import _lib
from pyloki_gb300.config import PulsarSearchConfig
from pyloki_gb300.ffa import DynamicProgramming, _cart_len
from pyloki_gb300.timeseries import TimeSeries


def pow2_length(n: int) -> int:
    """Largest power of two <= n (the length a series is truncated to)."""
    if n < 1:
        msg = "empty series"
        raise ValueError(msg)
    return 1 << (int(n).bit_length() - 1)


@dataclass
class Candidates:
    """Top-k final-level trials of one series: flat parameter indices of the
    final grid, their S/N (max over widths; float32 from the search, float64
    when re-scored) and the parameter values."""

    index: np.ndarray
    snr: np.ndarray
    params: np.ndarray
    snr_search: np.ndarray
    length: int


@dataclass
class TuneResult:
    chunk: int
    band_bytes: int
    ms_per_series: float
    tried: list = field(default_factory=list)


def _peak_bytes(cfg: PulsarSearchConfig, nbatch: int, band_bytes: int, elem: int) -> int:
    """Device bytes one banded search of ``nbatch`` series holds at its peak:
    two consecutive materialised levels, the two band buffers, the S/N."""
    n = cfg.niters_ffa
    prof = 2 * cfg.nbins * elem

    def lvl(level: int) -> int:
        nseg = nbatch * (cfg.nsamps // (cfg.bseg_brute * 2**level))
        return nseg * _cart_len(cfg.get_param_grid_count(level)) * prof

    mats = [lvl(0)] + [lvl(level) + lvl(level - 1) for level in range(1, max(1, n - 1))]
    snr = nbatch * _cart_len(cfg.get_param_grid_count(n)) * 4
    series = nbatch * cfg.nsamps * 8
    return max(mats) + 4 * band_bytes + 2 * snr + series


class Tuner:
    """Chooses (chunk, band_bytes) per search shape by timing on the device.

    Results are kept per key (length, grids, storage, device) in memory and,
    when ``path`` is given, in a JSON file that later runs read back.
    """

    def __init__(self, path: str | os.PathLike | None = None,
                 band_choices: Sequence[int] = (128 << 20, 384 << 20, 1 << 30)) -> None:
        self.path = path
        self.band_choices = tuple(band_choices)
        self.table: dict[str, dict] = {}
        if path is not None and os.path.exists(path):
            with open(path) as fh:
                self.table = json.load(fh)

    @staticmethod
    def key(cfg: PulsarSearchConfig, storage: str, device: torch.device) -> str:
        lim = ",".join(f"{a:.9g}:{b:.9g}" for a, b in np.asarray(cfg.param_limits))
        name = torch.cuda.get_device_name(device) if device.type == "cuda" else "cpu"
        return (f"{cfg.nsamps}|{cfg.tsamp:.9g}|{cfg.nbins}|{cfg.bseg_brute}|{lim}|"
                f"{cfg.score_widths.tolist()}|{storage}|{name}")

    def get(self, key: str) -> TuneResult | None:
        e = self.table.get(key)
        return None if e is None else TuneResult(e["chunk"], e["band_bytes"],
                                                 e["ms_per_series"], e.get("tried", []))

    def put(self, key: str, res: TuneResult) -> None:
        self.table[key] = {"chunk": res.chunk, "band_bytes": res.band_bytes,
                           "ms_per_series": res.ms_per_series, "tried": res.tried}
        if self.path is not None:
            tmp = f"{self.path}.tmp"
            with open(tmp, "w") as fh:
                json.dump(self.table, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.path)

    def tune(self, cfg: PulsarSearchConfig, storage: str, device: torch.device,
             n_series: int, mem_budget: int,
             time_fn: Callable[[int, int], float]) -> TuneResult:
        """``time_fn(chunk, band_bytes)`` returns ms for one pass of ``chunk``
        series. Chunks are powers of two up to ``n_series`` that fit in
        ``mem_budget``; bands are tried at the best chunk."""
        key = self.key(cfg, storage, device)
        hit = self.get(key)
        if hit is not None and hit.chunk <= max(1, n_series):
            return hit
        elem = 2 if storage == "bf16" else 4
        chunks = []
        c = 1
        while c <= max(1, n_series):
            if _peak_bytes(cfg, c, max(self.band_choices), elem) <= mem_budget:
                chunks.append(c)
            c *= 2
        if not chunks:
            msg = f"one series of {cfg.nsamps} samples does not fit in {mem_budget} bytes"
            raise MemoryError(msg)
        tried = []
        best = None
        base_band = self.band_choices[len(self.band_choices) // 2]
        for c in chunks:
            ms = time_fn(c, base_band) / c
            tried.append([c, base_band, ms])
            if best is None or ms < best[2]:
                best = [c, base_band, ms]
            elif ms > 1.15 * best[2]:
                break  # larger chunks past the optimum only cost memory
        for b in self.band_choices:
            if b == base_band:
                continue
            ms = time_fn(best[0], b) / best[0]
            tried.append([best[0], b, ms])
            if ms < best[2]:
                best = [best[0], b, ms]
        res = TuneResult(int(best[0]), int(best[1]), float(best[2]), tried)
        self.put(key, res)
        return res


class _ChunkGraph:
    """One chunk shape (length, nbatch): static input buffers, the search and
    its top-k captured in a CUDA graph."""

    def __init__(self, cfg: PulsarSearchConfig, nbatch: int, k: int, band_bytes: int,
                 storage: str, device: torch.device, use_graph: bool,
                 unit_variance: bool = False) -> None:
        self.cfg, self.nbatch, self.k = cfg, nbatch, k
        self.band_bytes, self.storage, self.device = band_bytes, storage, device
        self.ts_e = torch.zeros(nbatch * cfg.nsamps, dtype=torch.float32, device=device)
        self.ts_v = torch.ones(nbatch * cfg.nsamps, dtype=torch.float32, device=device)
        # the flag holds for every series this graph will see (decided by the
        # caller over all of them), not just the warm-up buffers
        self.dyp = DynamicProgramming(TimeSeries(self.ts_e, self.ts_v, cfg.tsamp), cfg,
                                      device=device, storage=storage, nbatch=nbatch,
                                      unit_variance=unit_variance)
        # grids referenced by raw pointers in the captured launches stay alive here
        self._grids = [self.dyp._grid(level) for level in range(cfg.niters_ffa + 1)]
        self.graph: torch.cuda.CUDAGraph | None = None
        self.launches_per_pass = 0
        self._eager()  # warm-up: builds grids, band plans, kernel attributes
        if use_graph:
            self._capture()

    def _body(self, check: bool) -> tuple[torch.Tensor, torch.Tensor]:
        self.dyp.reset()
        snr = self.dyp.search(mode=1, band_bytes=self.band_bytes, check=check)
        flat = snr.reshape(self.nbatch, -1)
        flat = torch.nan_to_num(flat, nan=float("-inf"))  # empty-bin trials are NaN
        vals, idx = torch.topk(flat, min(self.k, flat.shape[1]), dim=1)
        return vals, idx

    def _eager(self) -> tuple[torch.Tensor, torch.Tensor]:
        lib = _lib.load()
        before = lib.loki_launch_count()
        out = self._body(check=True)
        self.launches_per_pass = lib.loki_launch_count() - before
        return out

    def _capture(self) -> None:
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):  # a side-stream run before capture, as torch asks
            self._body(check=True)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self.vals, self.idx = self._body(check=False)

    def load(self, series: Sequence[TimeSeries]) -> None:
        n = self.cfg.nsamps
        for i in range(self.nbatch):
            ts = series[i] if i < len(series) else series[-1]
            e = torch.as_tensor(ts.ts_e)[:n]
            v = torch.as_tensor(ts.ts_v)[:n]
            self.ts_e[i * n:(i + 1) * n].copy_(e, non_blocking=True)
            self.ts_v[i * n:(i + 1) * n].copy_(v, non_blocking=True)

    def run(self) -> tuple[torch.Tensor, torch.Tensor]:
        if self.graph is None:
            return self._eager()
        self.graph.replay()
        return self.vals, self.idx


class BatchedSearch:
    """FFA search over many series (``cfg_for(length)`` gives each length's
    configuration), returning the top-``k`` candidates of every series.

    Parameters
    ----------
    series : sequence of TimeSeries
        Host or device series; each is truncated to ``pow2_length(len)``.
    cfg_for : callable
        ``cfg_for(nsamps) -> PulsarSearchConfig`` (one final segment per
        series: ``bseg_ffa == nsamps``).
    k : int
        Candidates kept per series (top S/N over widths; NaN trials last).
    storage : {"f32", "bf16"}
        Fold storage (``DynamicProgramming``).
    rescore : bool
        Re-score every kept candidate in FP64 from the samples
        (``DynamicProgramming.rescore``) and order by the FP64 S/N.
    use_graphs : bool
        Replay each chunk shape from a CUDA graph (eager launches otherwise).
    tuner : Tuner or None
        Chooses chunk and band sizes; None uses ``chunk`` and ``band_bytes``.
    mem_fraction : float
        Share of free device memory a chunk may use (tuner limit).
    """

    def __init__(self, series: Sequence[TimeSeries],
                 cfg_for: Callable[[int], PulsarSearchConfig], *, device=None, k: int = 16,
                 storage: str = "f32", rescore: bool = False, use_graphs: bool = True,
                 tuner: Tuner | None = None, chunk: int = 8, band_bytes: int = 1 << 30,
                 mem_fraction: float = 0.5) -> None:
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.series = list(series)
        self.cfg_for = cfg_for
        self.k, self.storage, self.rescore = k, storage, rescore
        self.use_graphs, self.tuner = use_graphs, tuner
        self.chunk, self.band_bytes, self.mem_fraction = chunk, band_bytes, mem_fraction
        # every series has ts_v all ones: the brute folds count instead of summing
        self.unit_variance = all(bool(np.all(np.asarray(
            ts.ts_v.cpu() if torch.is_tensor(ts.ts_v) else ts.ts_v) == 1.0)) for ts in self.series)
        self.groups: dict[int, list[int]] = {}
        for i, ts in enumerate(self.series):
            self.groups.setdefault(pow2_length(len(ts.ts_e)), []).append(i)
        self._cfgs = {n: cfg_for(n) for n in self.groups}
        for n, cfg in self._cfgs.items():
            if cfg.nsamps != n or cfg.nsamps != cfg.bseg_brute * 2**cfg.niters_ffa:
                msg = f"cfg_for({n}) must give nsamps {n} with one final segment"
                raise ValueError(msg)
        self._graphs: dict[tuple[int, int], _ChunkGraph] = {}
        self.plan: dict[int, TuneResult] = {}
        #: kernel launches of the last run() (library counter)
        self.launches = 0
        self.graph_launches = 0

    def trials(self) -> int:
        """Final-level trials of one pass over every series."""
        return sum(len(ids) * _cart_len(self._cfgs[n].get_param_grid_count(
            self._cfgs[n].niters_ffa)) for n, ids in self.groups.items())

    def _chunk_graph(self, n: int, nbatch: int, band_bytes: int) -> _ChunkGraph:
        key = (n, nbatch, band_bytes)
        g = self._graphs.get(key)
        if g is None:
            g = self._graphs[key] = _ChunkGraph(self._cfgs[n], nbatch, self.k, band_bytes,
                                                self.storage, self.device, self.use_graphs,
                                                self.unit_variance)
        return g

    def prepare(self) -> None:
        """Tune (if a tuner is set) and capture every chunk shape of the run."""
        free, _ = torch.cuda.mem_get_info(self.device)
        budget = int(free * self.mem_fraction)
        for n, ids in self.groups.items():
            cfg = self._cfgs[n]
            if self.tuner is not None:
                def time_fn(c: int, b: int, n=n) -> float:
                    g = _ChunkGraph(cfg, c, self.k, b, self.storage, self.device,
                                    use_graph=False, unit_variance=self.unit_variance)
                    g.load([self.series[i] for i in ids[:c]])
                    torch.cuda.synchronize(self.device)
                    t0 = torch.cuda.Event(enable_timing=True)
                    t1 = torch.cuda.Event(enable_timing=True)
                    t0.record()
                    g.run()
                    t1.record()
                    torch.cuda.synchronize(self.device)
                    del g
                    return t0.elapsed_time(t1)
                self.plan[n] = self.tuner.tune(cfg, self.storage, self.device, len(ids),
                                               budget, time_fn)
            else:
                self.plan[n] = TuneResult(max(1, min(self.chunk, len(ids))), self.band_bytes,
                                          float("nan"))
            c = min(self.plan[n].chunk, len(ids))
            self._chunk_graph(n, c, self.plan[n].band_bytes)
            rem = len(ids) % c
            if rem:
                self._chunk_graph(n, rem, self.plan[n].band_bytes)

    def run(self) -> list[Candidates]:
        """Search every series; candidates in input order."""
        if not self.plan:
            self.prepare()
        lib = _lib.load()
        before = lib.loki_launch_count()
        self.graph_launches = 0
        results: list[Candidates | None] = [None] * len(self.series)
        pending = []
        for n, ids in self.groups.items():
            c = min(self.plan[n].chunk, len(ids))
            for s0 in range(0, len(ids), c):
                part = ids[s0:s0 + c]
                g = self._chunk_graph(n, len(part), self.plan[n].band_bytes)
                g.load([self.series[i] for i in part])
                vals, idx = g.run()
                if g.graph is not None:
                    self.graph_launches += 1
                # FP64 re-scoring reads the chunk's series: before the next load
                snr64 = None
                if self.rescore:  # every kept candidate of the chunk in one launch
                    segs = torch.arange(len(part), device=self.device).repeat_interleave(
                        idx.shape[1])
                    snr64 = g.dyp.rescore(idx.reshape(-1), seg=segs).amax(dim=1).reshape(
                        idx.shape)
                pending.append((n, part, vals.clone(), idx.clone(), snr64, g))
        for n, part, vals, idx, snr64, g in pending:
            cfg = self._cfgs[n]
            fin = g.dyp._grid(cfg.niters_ffa)
            counts = fin.counts
            idx_h = idx.cpu().numpy()
            vals_h = vals.cpu().numpy()
            for j, i in enumerate(part):
                sel = idx_h[j]
                order = np.arange(len(sel))
                snr = vals_h[j].astype(np.float64)
                if snr64 is not None:
                    snr = snr64[j].cpu().numpy()
                    order = np.argsort(-np.nan_to_num(snr, nan=-np.inf), kind="stable")
                multi = np.stack(np.unravel_index(sel[order], counts), axis=1)
                params = np.stack([fin.param_arr[d][multi[:, d]]
                                   for d in range(cfg.nparams)], axis=1)
                results[i] = Candidates(sel[order], snr[order], params,
                                        vals_h[j][order], n)
        for g in {id(p[5]): p[5] for p in pending}.values():
            g.dyp.check_errors()
        self.launches = lib.loki_launch_count() - before + sum(
            p[5].launches_per_pass for p in pending if p[5].graph is not None)
        return results  # type: ignore[return-value]


def sequential_search(series: Sequence[TimeSeries],
                      cfg_for: Callable[[int], PulsarSearchConfig], *, device=None,
                      k: int = 16, band_bytes: int = 1 << 30) -> list[Candidates]:
    """The plain path: one ``DynamicProgramming.search`` per series, FP32,
    eager launches (the reference's one-series-per-call structure)."""
    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())
    out = []
    for ts in series:
        n = pow2_length(len(ts.ts_e))
        cfg = cfg_for(n)
        sub = TimeSeries(torch.as_tensor(ts.ts_e)[:n], torch.as_tensor(ts.ts_v)[:n], cfg.tsamp)
        dyp = DynamicProgramming(sub, cfg, device=dev)
        snr = dyp.search(mode=1, band_bytes=band_bytes).reshape(-1)
        vals, idx = torch.topk(torch.nan_to_num(snr, nan=float("-inf")), min(k, snr.numel()))
        fin = dyp._grid(cfg.niters_ffa)
        idx_h = idx.cpu().numpy()
        multi = np.stack(np.unravel_index(idx_h, fin.counts), axis=1)
        params = np.stack([fin.param_arr[d][multi[:, d]] for d in range(cfg.nparams)], axis=1)
        v = vals.cpu().numpy()
        out.append(Candidates(idx_h, v.astype(np.float64), params, v, n))
    return out


def cfg3_lengths(n_series: int, seed: int) -> np.ndarray:
    """Series lengths drawn uniformly in [2^20, 2^23] (seeded)."""
    rng = np.random.default_rng(seed)
    return rng.integers(2**20, 2**23 + 1, n_series)


__all__ = ["BatchedSearch", "Candidates", "Tuner", "cfg3_lengths", "pow2_length",
           "sequential_search"]

"""FFA dynamic programming on the GPU (drop-in for pyloki's ``ffa.py``).

``DynamicProgramming`` keeps the reference's interface (``ffa.py:196-435``):
``initialize`` brute-folds the series (``loki_brutefold``), ``execute`` runs
the DP levels (``loki_ffa_level``), and the grid properties are the
reference's. Folds live in HBM as torch tensors with pyloki's layout
``(nsegments, *param_counts, 2, nbins)``; with ``storage="bf16"`` the DP
levels store bfloat16 (FP32 arithmetic) and ``rescore`` recomputes the S/N of
retained candidates from the samples with FP64 sums.

``search`` is the memory-bounded path used by ``ffa_search``: the last level
is fused with normalisation and boxcar scoring (``loki_ffa_level_score``) and
never written; when the penultimate level is large, the last two levels run
in frequency bands whose penultimate fold fits in a small scratch buffer.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from pyloki_gb300 import _lib
from pyloki_gb300.config import PulsarSearchConfig
from pyloki_gb300.timeseries import TimeSeries

ffacoord_dtype = np.dtype(
    [("i_tail", np.uint32), ("shift_tail", np.float32),
     ("i_head", np.uint32), ("shift_head", np.float32)],
)
ffacoordfreq_dtype = np.dtype([("idx", np.uint32), ("shift", np.float32)])

_GIB = 1 << 30


def _cart_len(counts) -> int:
    return int(np.prod(np.asarray(counts, dtype=np.int64)))


class _Grid:
    """Per-level grid: counts and the parameter arrays, resident on the device."""

    def __init__(self, cfg: PulsarSearchConfig, level: int, device) -> None:
        self.level = level
        self.dparams = cfg.get_dparams(level)
        self.param_arr = cfg.get_param_arr(self.dparams)
        self.counts = np.array([len(p) for p in self.param_arr], dtype=np.int64)
        self.dev = [torch.from_numpy(np.ascontiguousarray(p, dtype=np.float64)).to(device)
                    for p in self.param_arr]
        # last-dimension grid as float2 (hi, lo): f == hi + lo to ~2^-48
        last = np.ascontiguousarray(self.param_arr[-1], dtype=np.float64)
        hi = last.astype(np.float32)
        lo = (last - hi.astype(np.float64)).astype(np.float32)
        self.split = torch.from_numpy(np.stack([hi, lo], axis=1).copy()).to(device)

    @property
    def size(self) -> int:
        return _cart_len(self.counts)


_GRID_CACHE: dict[tuple, _Grid] = {}


def _cfg_key(cfg: PulsarSearchConfig) -> tuple:
    return (cfg.nsamps, cfg.tsamp, cfg.nbins, cfg.eta, cfg.param_limits.tobytes(),
            cfg.bseg_brute, cfg.bseg_ffa)


def grid(cfg: PulsarSearchConfig, level: int, device) -> _Grid:
    """Device grid of one level, shared by every search with the same grids."""
    key = (_cfg_key(cfg), level, str(torch.device(device)))
    g = _GRID_CACHE.get(key)
    if g is None:
        if len(_GRID_CACHE) > 64:
            _GRID_CACHE.clear()
        g = _GRID_CACHE[key] = _Grid(cfg, level, device)
    return g


def level_desc(cfg: PulsarSearchConfig, cur: _Grid, prev: _Grid, nseg_in: int,
               out_win: tuple[int, int] | None = None,
               in_win: tuple[int, int] | None = None, *,
               storage: int = 0) -> _lib.LokiFFALevel:
    """Build the C descriptor of one DP level (optionally frequency-windowed).
    ``storage`` 0 keeps the folds in float32, 1 in bfloat16 (FP32 arithmetic)."""
    n = cfg.nparams
    d = _lib.LokiFFALevel()
    d.nparams = n
    d.nbins = cfg.nbins
    d.level = cur.level
    d.tseg_brute = cfg.tseg_brute
    for i in range(n):
        d.counts_cur[i] = int(cur.counts[i])
        d.counts_prev[i] = int(prev.counts[i])
        d.limits[i][0] = float(cfg.param_limits[i, 0])
        d.limits[i][1] = float(cfg.param_limits[i, 1])
        d.param_arr[i] = cur.dev[i].data_ptr()
    o0, ow = out_win if out_win is not None else (0, int(cur.counts[-1]))
    i0, iw = in_win if in_win is not None else (0, int(prev.counts[-1]))
    d.out_start, d.out_width = o0, ow
    d.in_start, d.in_width = i0, iw
    d.nseg_in = nseg_in
    d.last_split = cur.split.data_ptr()
    d.storage = storage
    return d


STORAGES = {"f32": (0, torch.float32), "bf16": (1, torch.bfloat16)}


class DynamicProgramming:
    """FFA dynamic programming (``ffa.py:196-435``) on one GB300.

    Parameters
    ----------
    ts_data : TimeSeries
        Input series (``ts_e``, ``ts_v`` float32).
    cfg : PulsarSearchConfig
        Search configuration (``use_fourier=False``: time-domain folds).
    device : torch.device or str, optional
        CUDA device, default the current one.
    storage : {"f32", "bf16"}
        Element type of the stored folds. ``"bf16"`` halves the HBM traffic of
        every DP level; the shift-add and the scoring still compute in FP32
        (each stored sum is rounded once to bfloat16); ``rescore`` gives the
        FP64 S/N of retained candidates.
    nbatch : int
        Number of equal-length series concatenated in ``ts_data``
        (``nbatch * cfg.nsamps`` samples). Their segments are stacked along
        the segment axis, so every level (and the fused final scoring) runs
        over all series in one launch; ``search`` then returns one S/N block
        per series. Each series must end in one final segment
        (``nsamps == bseg_brute * 2**niters_ffa``), so no segment pair spans
        two series.
    unit_variance : bool or None
        ``ts_v`` is all ones: the brute folds take the variance sums from
        sample counts (time domain) or once for all segments (Fourier
        domain), the same values. None (default) checks the series once at
        the first ``initialize``. True asserts the property without checking,
        for callers that reuse the object for other series (``BatchedSearch``
        decides over all of its series); with a ``ts_v`` that is not all ones
        the variance sums would be wrong.
    """

    def __init__(self, ts_data: TimeSeries, cfg: PulsarSearchConfig, *, device=None,
                 storage: str = "f32", nbatch: int = 1,
                 unit_variance: bool | None = None) -> None:
        if cfg.use_fourier and cfg.nbins % 2:
            msg = "the Fourier-domain FFA needs an even nbins (irfft length)"
            raise ValueError(msg)
        if storage not in STORAGES:
            msg = f"storage must be one of {sorted(STORAGES)}, got {storage!r}"
            raise ValueError(msg)
        if storage != "f32" and cfg.use_fourier:
            msg = "reduced-precision storage is for time-domain folds only"
            raise ValueError(msg)
        self._storage, self._fold_dtype = STORAGES[storage]
        self.storage = storage
        # ts_v all ones: the brute fold takes the variance sums from sample
        # counts. None: decided from the series at the first initialize.
        self._unit_var = unit_variance
        if nbatch < 1:
            msg = "nbatch must be >= 1"
            raise ValueError(msg)
        if nbatch > 1 and cfg.nsamps != cfg.bseg_brute * 2**cfg.niters_ffa:
            msg = ("batched series need one final segment each: nsamps == bseg_brute * "
                   f"2**niters_ffa ({cfg.nsamps} vs {cfg.bseg_brute} * 2**{cfg.niters_ffa})")
            raise ValueError(msg)
        if nbatch > 1 and cfg.use_fourier:
            msg = "batched series are for time-domain folds"
            raise ValueError(msg)
        self.nbatch = nbatch
        self._ts_dev: tuple[torch.Tensor, torch.Tensor] | None = None
        self._ts_data = ts_data
        self._cfg = cfg
        self._device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._lib = _lib.load()
        self._err = torch.zeros(1, dtype=torch.int32, device=self._device)
        self._data_type = np.complex64 if cfg.use_fourier else np.float32
        self._fold: torch.Tensor | None = None
        self._ffa_level = -1
        self.phase_scratch_bytes = _GIB
        #: kernels launched by this object (brute fold, levels, bands, scoring)
        self.launches = 0
        #: library launch counter at the phase marks of the last search()
        self.phase_marks: dict[str, int] = {}

    # ---- reference properties ------------------------------------------------
    @property
    def ts_data(self) -> TimeSeries:
        return self._ts_data

    @property
    def cfg(self) -> PulsarSearchConfig:
        return self._cfg

    @property
    def data_type(self):
        return self._data_type

    @property
    def device(self) -> torch.device:
        return self._device

    @property
    def fold(self) -> torch.Tensor:
        """Fold of the current level on the device, ``(nseg, *counts, 2, nbins)``."""
        if self._fold is None:
            msg = ("the fold of this level is not materialised (search() fuses the "
                   "last level with scoring); call execute() to materialise it")
            raise RuntimeError(msg)
        return self._fold

    @property
    def nsegments(self) -> int:
        return self.nbatch * (self.cfg.nsamps // (self.cfg.bseg_brute * 2**self.ffa_level))

    @property
    def nbins(self) -> int:
        return self.cfg.nbins

    @property
    def ffa_level(self) -> int:
        return self._ffa_level

    def _grid(self, level: int) -> _Grid:
        return grid(self.cfg, level, self._device)

    @property
    def dparams(self) -> np.ndarray:
        return self._grid(self.ffa_level).dparams

    @property
    def dparams_actual(self) -> np.ndarray:
        return self.cfg.get_dparams_actual(self.ffa_level)

    @property
    def param_arr(self) -> list[np.ndarray]:
        return self._grid(self.ffa_level).param_arr

    @property
    def param_grid_count(self) -> np.ndarray:
        return self.cfg.get_param_grid_count(self.ffa_level)

    @property
    def param_arr_dict(self) -> dict[str, np.ndarray]:
        names = self.cfg.param_names
        return {f"{names[i]}": p for i, p in enumerate(self.param_arr)}

    @property
    def nparam_vol(self) -> int:
        return int(np.prod([len(p) for p in self.param_arr])) if self.param_arr else 0

    @property
    def leaves_lb(self) -> float:
        return np.round(np.log2(self.nparam_vol), 2)

    @property
    def tseg(self) -> float:
        return self.cfg.tseg_brute * 2**self.ffa_level

    def _stream(self) -> int:
        return _lib.stream_ptr(torch.cuda.current_stream(self._device))

    # ---- level 0: brute fold -------------------------------------------------
    def initialize(self) -> None:
        """Brute-fold the series at the level-0 grid (``ffa.py:305-329``)."""
        cfg = self.cfg
        g0 = self._grid(0)
        if cfg.nparams > 1:
            for ip in range(cfg.nparams - 1):
                if len(g0.param_arr[ip]) > 1:
                    msg = (f"param_arr has {len(g0.param_arr[ip])} values, "
                           "should have only one")
                    raise ValueError(msg)
        freqs = g0.param_arr[-1]
        if not np.all(np.isfinite(freqs)) or np.any(freqs <= 0):
            msg = "Frequency must be positive."
            raise ValueError(msg)
        dev = self._device
        ts_e = torch.as_tensor(self.ts_data.ts_e).to(dev, non_blocking=True)
        ts_v = torch.as_tensor(self.ts_data.ts_v).to(dev, non_blocking=True)
        if ts_e.numel() != self.nbatch * cfg.nsamps or ts_v.numel() != ts_e.numel():
            msg = (f"expected {self.nbatch} x {cfg.nsamps} samples in ts_e and ts_v, got "
                   f"{ts_e.numel()} and {ts_v.numel()}")
            raise ValueError(msg)
        self._ts_dev = (ts_e, ts_v)
        t_ref = 0.0 if cfg.nparams == 1 else cfg.bseg_brute * cfg.tsamp / 2
        if self._unit_var is None:
            src = self.ts_data.ts_v
            self._unit_var = (bool((ts_v == 1.0).all()) if torch.is_tensor(src)
                              else bool(np.all(np.asarray(src) == 1.0)))
        if cfg.use_fourier:  # core/fold.py:395-481,572-614
            nseg = ts_e.numel() // cfg.bseg_brute
            nfreq = g0.dev[-1].numel()
            nbf = cfg.nbins // 2 + 1
            fold = torch.empty((nseg, nfreq, 2, nbf), dtype=torch.complex64, device=dev)
            _lib.check(self._lib.loki_brutefold_complex(
                _lib.ptr(ts_e), 0 if self._unit_var else _lib.ptr(ts_v), ts_e.numel(),
                _lib.ptr(g0.dev[-1]), nfreq,
                cfg.bseg_brute, cfg.nbins, cfg.tsamp, t_ref, _lib.ptr(fold), self._stream()))
            self.launches += 1
            self._fold = fold.reshape(nseg, *([1] * (cfg.nparams - 1)), nfreq, 2, nbf)
            self._err.zero_()
            self._ffa_level = 0
            return
        self._fold, nl = _brutefold(ts_e, ts_v, g0.dev[-1], cfg.bseg_brute, cfg.nbins,
                                    cfg.tsamp, 0.0 if cfg.nparams == 1 else
                                    cfg.bseg_brute * cfg.tsamp / 2,
                                    scratch_bytes=self.phase_scratch_bytes,
                                    unit_variance=self._unit_var)
        self.launches += nl
        nseg, nfreq = self._fold.shape[:2]
        if self._storage:
            low = torch.empty(self._fold.shape, dtype=self._fold_dtype, device=dev)
            _lib.check(self._lib.loki_f32_to_bf16(_lib.ptr(self._fold), self._fold.numel(),
                                                  _lib.ptr(low), self._stream()))
            self.launches += 1
            self._fold = low
        self._fold = self._fold.reshape(nseg, *([1] * (cfg.nparams - 1)), nfreq, 2,
                                        cfg.nbins)
        self._err.zero_()
        self._ffa_level = 0

    # ---- DP levels -----------------------------------------------------------
    def execute(self, *, show_progress: bool = False) -> None:
        """Run every DP level, materialising each fold (``ffa.py:331-347``)."""
        for _ in range(self.cfg.niters_ffa - self.ffa_level):
            self._execute_iter()
        _lib.check_dev_err(self._err)

    def _execute_iter(self) -> None:
        cur = self._grid(self.ffa_level + 1)
        prev = self._grid(self.ffa_level)
        nseg_in = self.nsegments
        fold_in = self.fold
        if self.cfg.use_fourier:  # shift_add_complex (core/common.py:344-372)
            nbf = self.nbins // 2 + 1
            desc = level_desc(self.cfg, cur, prev, nseg_in)
            plan = torch.empty((cur.size, 4), dtype=torch.int32, device=self._device)
            _lib.check(self._lib.loki_ffa_plan(desc, _lib.ptr(plan), _lib.ptr(self._err),
                                               self._stream()))
            out = torch.empty((nseg_in // 2, cur.size, 2, nbf), dtype=torch.complex64,
                              device=self._device)
            _lib.check(self._lib.loki_ffa_level_complex(desc, _lib.ptr(plan), _lib.ptr(fold_in),
                                                        _lib.ptr(out), self._stream()))
            self.launches += 2
            self._fold = out.reshape(nseg_in // 2, *cur.counts.tolist(), 2, nbf)
            self._ffa_level += 1
            return
        out = torch.empty((nseg_in // 2, cur.size, 2, self.nbins), dtype=self._fold_dtype,
                          device=self._device)
        desc = level_desc(self.cfg, cur, prev, nseg_in, storage=self._storage)
        _lib.check(self._lib.loki_ffa_level(desc, _lib.ptr(fold_in), _lib.ptr(out),
                                            _lib.ptr(self._err), self._stream()))
        self.launches += 1
        self._fold = out.reshape(nseg_in // 2, *cur.counts.tolist(), 2, self.nbins)
        self._ffa_level += 1

    def get_fold_norm(self, iseg: int = 0, param_idx: tuple | None = None) -> torch.Tensor:
        """``fold[iseg][..., 0, :] / sqrt(fold[iseg][..., 1, :])`` (``ffa.py:382-411``)."""
        fold = self.fold[iseg]
        if param_idx is not None:
            idx = tuple(int(i) for i in param_idx)[-(fold.ndim - 2):]
            fold = fold[idx]
        lead = fold.shape[:-2]
        flat = fold.reshape(-1, 2, fold.shape[-1]).contiguous()
        if flat.dtype == torch.bfloat16:
            flat = flat.float()
        out = torch.empty((flat.shape[0], self.nbins), dtype=torch.float32,
                          device=self._device)
        if self.cfg.use_fourier:  # irfft, then e / sqrt(v)
            _lib.check(self._lib.loki_fold_norm_complex(_lib.ptr(flat), flat.shape[0],
                                                        self.nbins, _lib.ptr(out),
                                                        self._stream()))
        else:
            _lib.check(self._lib.loki_fold_norm(_lib.ptr(flat), flat.shape[0], self.nbins,
                                                _lib.ptr(out), self._stream()))
        self.launches += 1
        return out.reshape(*lead, self.nbins)

    def get_complexity(self) -> list[int]:
        return [_cart_len(self.cfg.get_param_grid_count(lvl))
                for lvl in range(self.cfg.niters_ffa + 1)]

    def rescore(self, cand, widths=None, stdnoise: float = 1.0, *, seg=0,
                level: int | None = None,
                return_profiles: bool = False) -> torch.Tensor | tuple[torch.Tensor, torch.Tensor]:
        """FP64 S/N ``(ncand, nwidths)`` of candidates given as flat parameter
        indices of ``level`` (default the final level), their folds rebuilt
        from the samples with FP64 sums (``loki_ffa_rescore``). ``seg`` is one
        segment of that level for every candidate, or one per candidate (with
        ``nbatch`` series and the final level, segment i is series i). With
        ``return_profiles`` also the FP64 folds ``(ncand, 2, nbins)``."""
        if self._ts_dev is None:
            msg = "rescore needs the series on the device: call initialize() or search() first"
            raise RuntimeError(msg)
        cfg = self.cfg
        level = cfg.niters_ffa if level is None else int(level)
        if not 1 <= level <= min(cfg.niters_ffa, _lib.MAX_RESCORE_LEVELS):
            msg = f"level {level} outside 1..{min(cfg.niters_ffa, _lib.MAX_RESCORE_LEVELS)}"
            raise ValueError(msg)
        widths = cfg.score_widths if widths is None else np.asarray(widths, np.int64)
        spec = _lib.score_spec(widths, cfg.nbins, stdnoise, mode=0)
        cand = torch.as_tensor(cand, dtype=torch.int64).reshape(-1).to(self._device)
        segs = None
        if not np.isscalar(seg):
            segs = torch.as_tensor(seg, dtype=torch.int64).reshape(-1).to(self._device)
            if segs.numel() != cand.numel():
                msg = "seg must be one segment or one per candidate"
                raise ValueError(msg)
            seg = 0
        descs = (_lib.LokiFFALevel * level)()
        for lvl in range(1, level + 1):
            nseg_in = cfg.nsamps // (cfg.bseg_brute * 2 ** (lvl - 1))
            descs[lvl - 1] = level_desc(cfg, self._grid(lvl), self._grid(lvl - 1), nseg_in)
        snr = torch.empty((cand.numel(), len(widths)), dtype=torch.float64, device=self._device)
        prof = (torch.empty((cand.numel(), 2, cfg.nbins), dtype=torch.float64,
                            device=self._device) if return_profiles else None)
        ts_e, ts_v = self._ts_dev
        f0 = self._grid(0).dev[-1]
        _lib.check(self._lib.loki_ffa_rescore(
            descs, level, _lib.ptr(ts_e), _lib.ptr(ts_v), ts_e.numel(), cfg.tsamp,
            cfg.bseg_brute, _lib.ptr(f0), f0.numel(), _lib.ptr(cand), _lib.ptr(segs),
            cand.numel(), int(seg), spec, _lib.ptr(snr), _lib.ptr(prof), self._stream()))
        self.launches += 1
        return (snr, prof) if return_profiles else snr

    # ---- fused, memory-bounded search ---------------------------------------
    def level_bytes(self, level: int) -> int:
        nseg = self.nbatch * (self.cfg.nsamps // (self.cfg.bseg_brute * 2**level))
        return (nseg * _cart_len(self.cfg.get_param_grid_count(level)) * 2 * self.nbins
                * self._elem_bytes)

    @property
    def _elem_bytes(self) -> int:
        return 2 if self._storage else 4

    def search(self, widths=None, stdnoise: float = 1.0, *, mode: int = 0,
               banded: bool | None = None, band_bytes: int = 1 << 30,
               final: str = "auto", norm: str = "exact",
               phase_events: list | None = None, check: bool = True) -> torch.Tensor:
        """S/N of every final-level parameter set (segment 0 of each series),
        never writing the final fold. Returns ``(*counts_final, nwidths)`` (or
        ``counts_final`` for ``mode=1``, the max over widths), with a leading
        series axis when ``nbatch > 1``. ``phase_events``, if given, receives
        ``(name, cuda.Event)`` marks recorded on the launch stream after the
        brute fold, the materialised levels and the final levels. ``check=False``
        leaves the device error word unread (no host synchronisation, as CUDA
        graph capture requires); read it later with ``check_errors``.

        ``final`` picks how the last levels run: ``"tiled"`` fuses the last
        two into one persistent launch that builds the penultimate rows of
        each tile in shared memory (64 bins, widths 1, 2, 4, ...);
        ``"banded"`` writes the penultimate level band by band to a scratch
        buffer; ``"level"`` materialises the penultimate level and fuses only
        the final one with scoring. ``"auto"`` takes the tiled path where it
        applies, else banded when the penultimate level is above
        ``8 * band_bytes``, else level. ``banded=True`` / ``False`` (with
        ``final="auto"``) asks for banded / level. ``norm`` applies to the
        tiled path: ``"exact"`` divides by the correctly rounded square root
        (S/N bit-identical to the reference); ``"fast"`` multiplies by the
        reciprocal square root (S/N within 1e-5 of it, relative to
        max(|S/N|, 1))."""
        if final not in ("auto", "tiled", "banded", "level"):
            msg = f"final must be 'auto', 'tiled', 'banded' or 'level', got {final!r}"
            raise ValueError(msg)
        if norm not in ("exact", "fast"):
            msg = f"norm must be 'exact' or 'fast', got {norm!r}"
            raise ValueError(msg)
        cfg = self.cfg
        n = cfg.niters_ffa
        widths = cfg.score_widths if widths is None else np.asarray(widths, np.int64)
        spec = _lib.score_spec(widths, cfg.nbins, stdnoise, mode=mode)
        spec.nseg = self.nbatch
        nout = len(widths) if mode == 0 else 1

        def mark(name: str) -> None:
            self.phase_marks[name] = self._lib.loki_launch_count()
            if phase_events is not None:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(torch.cuda.current_stream(self._device))
                phase_events.append((name, ev))

        mark("start")
        if self.ffa_level < 0:
            self.initialize()
        if self.ffa_level != 0:
            msg = "search() starts from the level-0 fold; call initialize() first"
            raise RuntimeError(msg)
        mark("brutefold")
        fin = self._grid(n)
        if cfg.use_fourier:  # every level materialised, then irfft norm + boxcar
            self.execute()
            mark("levels")
            from pyloki_gb300.scoring import boxcar_snr_nd

            snr = boxcar_snr_nd(self.get_fold_norm(), widths, stdnoise)
            if mode != 0:
                snr = snr.amax(dim=-1)
            mark("final")
            return snr
        snr = torch.empty((self.nbatch, fin.size, nout), dtype=torch.float32,
                          device=self._device)
        widths_arr = np.asarray(widths, np.int64)
        tiled_ok = (n >= 2 and cfg.nbins == 64 and len(widths_arr) <= 6
                    and np.array_equal(widths_arr, 2 ** np.arange(len(widths_arr))))
        if final == "tiled" and not tiled_ok:
            msg = "the tiled final levels need >= 2 levels, 64 bins and widths 1, 2, 4, ..."
            raise ValueError(msg)
        if final == "auto":
            if banded is not None:
                final = "banded" if banded else "level"
            elif tiled_ok:
                final = "tiled"
            else:
                final = ("banded" if n >= 2 and self.level_bytes(n - 1) > 8 * band_bytes
                         else "level")
        if final == "banded" and n < 2:
            final = "level"
        self.final_path = final
        tiled = final == "tiled"
        banded = final == "banded"
        last_mat = n - 2 if (banded or tiled) else n - 1
        while self.ffa_level < last_mat:
            self._execute_iter()
        mark("levels")
        if tiled:
            self._search_tiled(fin, spec, snr, fast=norm == "fast")
        elif not banded:
            prev = self._grid(n - 1)
            desc = level_desc(cfg, fin, prev, self.nsegments, storage=self._storage)
            _lib.check(self._lib.loki_ffa_level_score(
                desc, _lib.ptr(self.fold), spec, _lib.ptr(snr), _lib.ptr(self._err),
                self._stream()))
            self.launches += 1
        else:
            self._search_banded(fin, spec, snr, band_bytes)
        mark("final")
        self._fold = None
        self._ffa_level = n
        if check:
            _lib.check_dev_err(self._err)
        shape = (*fin.counts.tolist(), nout) if mode == 0 else tuple(fin.counts.tolist())
        if self.nbatch > 1:
            shape = (self.nbatch, *shape)
        return snr.reshape(shape)

    def check_errors(self) -> None:
        """Raise if a kernel of this object flagged a device error (reads the
        error word: one host synchronisation)."""
        _lib.check_dev_err(self._err)

    def reset(self) -> None:
        """Return to the state before ``initialize`` (grids and device series
        stay), so that ``search`` can run again on the same buffers."""
        self._fold = None
        self._ffa_level = -1

    def band_plan(self, band_bytes: int) -> tuple[int, np.ndarray, np.ndarray]:
        """Frequency bands for the last two levels: (final band width, lo, hi)
        where [lo[k], hi[k]] is the penultimate frequency window of band k."""
        cfg = self.cfg
        n = cfg.niters_ffa
        fin, pen = self._grid(n), self._grid(n - 1)
        nseg_pen = self.nbatch * (cfg.nsamps // (cfg.bseg_brute * 2 ** (n - 1)))
        other_pen = _cart_len(pen.counts[:-1])
        row = nseg_pen * other_pen * 2 * cfg.nbins * self._elem_bytes
        w_pen = max(64, band_bytes // row)
        width = max(32, int(2 * w_pen * 0.75))
        width = min(width, int(fin.counts[-1]))
        desc = level_desc(cfg, fin, pen, nseg_pen)
        key = (_cfg_key(cfg), band_bytes, self._storage, self.nbatch, str(self._device))
        if key in _BAND_CACHE:
            return _BAND_CACHE[key]
        for _ in range(8):
            nb = math.ceil(int(fin.counts[-1]) / width)
            lo = torch.empty(nb, dtype=torch.int64, device=self._device)
            hi = torch.empty(nb, dtype=torch.int64, device=self._device)
            _lib.check(self._lib.loki_ffa_band_windows(desc, width, _lib.ptr(lo), _lib.ptr(hi),
                                                       self._stream()))
            self.launches += 1
            lo_h, hi_h = lo.cpu().numpy(), hi.cpu().numpy()
            _BAND_CACHE[key] = (width, lo_h, hi_h)
            if (hi_h - lo_h + 1).max() <= 2 * w_pen or width <= 32:
                return width, lo_h, hi_h
            width = max(32, width // 2)
        return width, lo_h, hi_h

    def _search_tiled(self, fin: _Grid, spec, snr: torch.Tensor, *, fast: bool) -> None:
        cfg = self.cfg
        n = cfg.niters_ffa
        pen, pp = self._grid(n - 1), self._grid(n - 2)
        nseg_pp = self.nsegments
        d_pen = level_desc(cfg, pen, pp, nseg_pp, storage=self._storage)
        d_fin = level_desc(cfg, fin, pen, nseg_pp // 2, storage=self._storage)
        nbytes = int(self._lib.loki_ffa_final_tiled_scratch(d_pen, d_fin))
        if nbytes <= 0:
            msg = "invalid tiled level descriptors"
            raise ValueError(msg)
        scratch = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=self._device)
        before = self._lib.loki_launch_count()
        _lib.check(self._lib.loki_ffa_final_tiled(
            d_pen, d_fin, _lib.ptr(self.fold), _lib.ptr(scratch), scratch.numel() * 8, spec,
            1 if fast else 0, _lib.ptr(snr), _lib.ptr(self._err), self._stream()))
        self.launches += self._lib.loki_launch_count() - before

    def _search_banded(self, fin: _Grid, spec, snr: torch.Tensor, band_bytes: int) -> None:
        cfg = self.cfg
        n = cfg.niters_ffa
        pen, pp = self._grid(n - 1), self._grid(n - 2)
        nseg_pp = self.nsegments
        nseg_pen = nseg_pp // 2
        width, lo, hi = self.band_plan(band_bytes)
        wmax = int((hi - lo + 1).max())
        d_pen = level_desc(cfg, pen, pp, nseg_pp, storage=self._storage)
        d_fin = level_desc(cfg, fin, pen, nseg_pen, storage=self._storage)
        nfl = int(self._lib.loki_ffa_final_banded_scratch(d_pen, d_fin, wmax))
        if nfl <= 0:
            msg = "invalid banded level descriptors"
            raise ValueError(msg)
        scratch = torch.empty(nfl, dtype=torch.float32, device=self._device)
        lo = np.ascontiguousarray(lo, np.int64)
        hi = np.ascontiguousarray(hi, np.int64)
        before = self._lib.loki_launch_count()
        _lib.check(self._lib.loki_ffa_final_banded(
            d_pen, d_fin, width, lo.ctypes.data, hi.ctypes.data, _lib.ptr(self.fold),
            _lib.ptr(scratch), scratch.numel(), spec, _lib.ptr(snr), _lib.ptr(self._err),
            self._stream()))
        self.launches += self._lib.loki_launch_count() - before


_BAND_CACHE: dict[tuple, tuple] = {}


def _brutefold(ts_e, ts_v, freqs, segment_len, nbins, tsamp, t_ref=0.0, *,
               scratch_bytes=_GIB, unit_variance: bool = False) -> tuple[torch.Tensor, int]:
    """Brute fold plus the number of kernels it launched."""
    lib = _lib.load()
    before = lib.loki_launch_count()
    fold = brutefold(ts_e, ts_v, freqs, segment_len, nbins, tsamp, t_ref,
                     scratch_bytes=scratch_bytes, unit_variance=unit_variance)
    return fold, lib.loki_launch_count() - before


def brutefold(ts_e: torch.Tensor, ts_v: torch.Tensor, freqs: torch.Tensor, segment_len: int,
              nbins: int, tsamp: float, t_ref: float = 0.0, *,
              scratch_bytes: int = _GIB, unit_variance: bool = False) -> torch.Tensor:
    """Fold ``(nsegments, nfreqs, 2, nbins)`` (``core/fold.py:108-171``).
    ``scratch_bytes`` bounds the phase map and chain layout; frequencies
    beyond it are folded in chunks. ``unit_variance``: the caller asserts
    ``ts_v`` is all ones, and the variance sums come from sample counts (the
    same values)."""
    lib = _lib.load()
    nsamps = ts_e.numel()
    nseg = math.ceil(nsamps / segment_len)
    nfreq = freqs.numel()
    elem = 1 if nbins <= 256 else 2
    need = int(lib.loki_brutefold_scratch_bytes(nfreq, segment_len, nbins))
    scratch = torch.empty(min(need, max(scratch_bytes, segment_len * elem)),
                          dtype=torch.uint8, device=ts_e.device)
    fold = torch.empty((nseg, nfreq, 2, nbins), dtype=torch.float32, device=ts_e.device)
    stream = _lib.stream_ptr(torch.cuda.current_stream(ts_e.device))
    if unit_variance:
        _lib.check(lib.loki_brutefold_unit_variance(
            _lib.ptr(ts_e), nsamps, _lib.ptr(freqs), nfreq, segment_len, nbins, tsamp, t_ref,
            _lib.ptr(scratch), scratch.numel(), _lib.ptr(fold), stream))
        return fold
    _lib.check(lib.loki_brutefold(_lib.ptr(ts_e), _lib.ptr(ts_v), nsamps, _lib.ptr(freqs),
                                  nfreq, segment_len, nbins, tsamp, t_ref,
                                  _lib.ptr(scratch), scratch.numel(), _lib.ptr(fold),
                                  stream))
    return fold


def brutefold_bucketed(ts_e: torch.Tensor, ts_v: torch.Tensor, freqs: torch.Tensor,
                       segment_len: int, nbins: int, tsamp: float,
                       t_ref: float = 0.0) -> torch.Tensor:
    """``core/fold.py:174-276``. The reference gathers each (frequency, bin)
    bucket and sums it in sample order: the same sums, in the same order, as
    ``brutefold``, which computes them. Like the reference it requires whole
    segments."""
    if ts_e.numel() % segment_len:
        msg = "The number of samples must be a multiple of the segment length."
        raise ValueError(msg)
    return brutefold(ts_e, ts_v, freqs, segment_len, nbins, tsamp, t_ref)


def brutefold_complex_oversampled(ts_e: torch.Tensor, ts_v: torch.Tensor, freqs: torch.Tensor,
                                  segment_len: int, nbins: int, tsamp: float,
                                  t_ref: float = 0.0,
                                  oversample_factor: int = 4) -> torch.Tensor:
    """``core/fold.py:484-524``: the fold on ``nbins * oversample_factor``
    bins, transformed along the bins (cuFFT) and cut to the first
    ``nbins // 2 + 1`` coefficients, complex64 ``(nseg, nfreq, 2, nbins//2+1)``."""
    fine = brutefold_bucketed(ts_e, ts_v, freqs, segment_len, nbins * oversample_factor, tsamp,
                              t_ref)
    return torch.fft.rfft(fine, dim=-1)[..., :nbins // 2 + 1].to(torch.complex64).contiguous()


class FFAPlan:
    """Per-level coordinate plan (``ffa.py:53-193``), resolved on the GPU."""

    def __init__(self, cfg: PulsarSearchConfig, *, device=None) -> None:
        self._cfg = cfg
        self._device = torch.device(device or "cuda")
        self.n_params = cfg.nparams
        self.n_levels = cfg.niters_ffa + 1
        self.params = [cfg.get_param_arr(cfg.get_dparams(lvl)) for lvl in range(self.n_levels)]
        self.param_counts = np.array(
            [cfg.get_param_grid_count(lvl) for lvl in range(self.n_levels)], dtype=np.int32)
        self.ncoords = np.array([_cart_len(c) for c in self.param_counts], dtype=np.int64)

    @property
    def cfg(self) -> PulsarSearchConfig:
        return self._cfg

    def resolve_level(self, level: int) -> np.ndarray:
        """Plan of one level (>= 1) as an ``ffacoord_dtype`` array."""
        lib = _lib.load()
        cur = _Grid(self.cfg, level, self._device)
        prev = _Grid(self.cfg, level - 1, self._device)
        nseg_in = self.cfg.nsamps // (self.cfg.bseg_brute * 2 ** (level - 1))
        desc = level_desc(self.cfg, cur, prev, nseg_in)
        coords = torch.empty((cur.size, 4), dtype=torch.int32, device=self._device)
        err = torch.zeros(1, dtype=torch.int32, device=self._device)
        stream = _lib.stream_ptr(torch.cuda.current_stream(self._device))
        _lib.check(lib.loki_ffa_plan(desc, _lib.ptr(coords), _lib.ptr(err), stream))
        _lib.check_dev_err(err)
        return coords.cpu().numpy().view(ffacoord_dtype).reshape(-1)

    def resolve_coordinates(self) -> list[np.ndarray]:
        """Plans of levels 1..n (level 0 is the brute fold and has no plan)."""
        return [np.zeros(0, ffacoord_dtype)] + [
            self.resolve_level(lvl) for lvl in range(1, self.n_levels)]

    def resolve_coordinates_freq(self) -> list[np.ndarray]:
        if self.n_params != 1:
            msg = "resolve_coordinates_freq is only supported for single parameter"
            raise ValueError(msg)
        out = [np.zeros(0, ffacoordfreq_dtype)]
        for lvl in range(1, self.n_levels):
            c = self.resolve_level(lvl)
            f = np.empty(len(c), ffacoordfreq_dtype)
            f["idx"] = c["i_head"]
            f["shift"] = c["shift_head"]
            out.append(f)
        return out


def compute_ffa(tseries: TimeSeries, search_cfg: PulsarSearchConfig, *, quiet: bool = False,
                show_progress: bool = False) -> torch.Tensor:
    """Final FFA fold (``ffa.py:438-467``), materialised on the device."""
    dyp = DynamicProgramming(tseries, search_cfg)
    dyp.initialize()
    dyp.execute(show_progress=show_progress)
    return dyp.fold

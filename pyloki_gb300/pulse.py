"""Synthetic pulsar series generated on the device
(``simulation/pulse.py``: ``build_cdf_lut`` 13-35, ``generate_pulse_template``
38-68, ``calibrate_scale_on_folds`` 71-118, ``PulseSignalConfig`` 121-432).

``PulseSignalConfig.generate`` follows the reference step by step (proper
time of the modulation model, CDF-table template, unit white noise, folds at
the pulse period, noise scale from the off-pulse bins, damped Newton
calibration of the signal scale on the folds, float32 output), but runs every
per-sample step in CUDA kernels (``csrc/pulse.cu``) and takes a batch of
injections in one pass (``generate_injections``), for training and
injection-recovery sets of thousands of series.

Differences from the reference, all deliberate:
- noise comes from a seeded counter-based generator (Philox-4x32-10 with the
  Box-Muller transform) instead of numpy's unseeded default generator, or from
  a caller-supplied array (``noise=``), which reproduces the reference's
  output exactly given the reference's draws;
- the calibration folds are exact sums (fixed point) rather than float32
  running sums, so the scales can differ from the reference's by float32
  rounding of the folds; the same seed always gives the same series;
- the series has exactly ``nsamps`` samples (the reference's
  ``np.arange(0, tobs, dt)`` can give one more, which it then rejects).
"""

from __future__ import annotations

from dataclasses import dataclass, field, fields, replace

import numpy as np
import torch

from pyloki_gb300 import _lib
from pyloki_gb300.modulate import type_to_mods
from pyloki_gb300.timeseries import TimeSeries

SHAPES = ("boxcar", "gaussian", "von_mises")


def build_cdf_lut(shape: str, width: float, pos: float, ngrid: int = 4096) -> np.ndarray:
    """Cumulative distribution of the pulse over one turn on ``ngrid`` phases
    plus the wrapped first value (float32, ``ngrid + 1`` entries)."""
    from scipy import stats

    phase = np.linspace(0.0, 1.0, ngrid, endpoint=False)
    if shape == "boxcar":
        rv = stats.uniform(loc=pos, scale=width)
    elif shape == "gaussian":
        rv = stats.norm(loc=pos, scale=width / (2 * np.sqrt(2 * np.log(10))))
    elif shape == "von_mises":
        kappa = np.log(2.0) / (2.0 * np.sin(np.pi * width / 2.0) ** 2)
        rv = stats.vonmises(loc=pos, kappa=kappa)
    else:
        msg = f"Unknown shape: {shape}"
        raise ValueError(msg)
    cdf = rv.cdf(phase).astype(np.float64)
    return np.concatenate([cdf, cdf[:1]]).astype(np.float32)


def cdf_tables(keys) -> dict:
    """``build_cdf_lut`` for many (shape, width, pos, ngrid) keys with one
    scipy call per (shape, ngrid) group. The shape parameters come from the
    same scalar expressions and the distributions are evaluated element by
    element, so every table equals its ``build_cdf_lut``."""
    from scipy import stats

    groups: dict = {}
    for key in keys:
        groups.setdefault((key[0], int(key[3])), []).append(key)
    out = {}
    for (shape, ngrid), ks in groups.items():
        phase = np.linspace(0.0, 1.0, ngrid, endpoint=False)[None, :]
        pos = np.array([float(k[2]) for k in ks])[:, None]
        if shape == "boxcar":
            cdf = stats.uniform.cdf(phase, loc=pos,
                                    scale=np.array([float(k[1]) for k in ks])[:, None])
        elif shape == "gaussian":
            sig = [float(k[1]) / (2 * np.sqrt(2 * np.log(10))) for k in ks]
            cdf = stats.norm.cdf(phase, loc=pos, scale=np.array(sig)[:, None])
        elif shape == "von_mises":
            kap = [np.log(2.0) / (2.0 * np.sin(np.pi * float(k[1]) / 2.0) ** 2) for k in ks]
            cdf = stats.vonmises.cdf(phase, np.array(kap)[:, None], loc=pos)
        else:
            msg = f"Unknown shape: {shape}"
            raise ValueError(msg)
        cdf = np.asarray(cdf, dtype=np.float64)
        cdf = np.concatenate([cdf, cdf[:, :1]], axis=1).astype(np.float32)
        for k, row in zip(ks, cdf):
            out[k] = row
    return out


def _seeds(seed: int | None, n: int) -> np.ndarray:
    ss = np.random.SeedSequence(seed)
    return np.array([c.generate_state(1, np.uint64)[0] for c in ss.spawn(n)], dtype=np.uint64)


def _device(device) -> torch.device:
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


@dataclass
class PulseSignalConfig:
    """A pulsar signal: period (s), sampling (s), length, folded S/N, duty
    cycle (full width at a tenth of the maximum, in turns) and a time
    modulation ``mod_type`` with ``mod_kwargs`` about ``mod_tref`` (default
    the middle of the observation)."""

    period: float
    dt: float
    nsamps: int = 2**21
    snr: float = 100
    ducy: float = 0.1
    ds: float = 1.0
    mod_type: str = "derivative"
    mod_kwargs: dict = field(default_factory=dict)
    mod_tref: float | None = None

    def __post_init__(self) -> None:
        if self.mod_type not in type_to_mods:
            msg = f"Unknown modulation: {self.mod_type}"
            raise ValueError(msg)
        self._mod_func = type_to_mods[self.mod_type](**self.mod_kwargs)
        if self.ducy <= 0 or self.ducy >= 1:
            msg = f"Duty cycle ({self.ducy}) should be in (0, 1)"
            raise ValueError(msg)
        if self.mod_tref is None:
            self.mod_tref = self.tobs / 2

    @property
    def freq(self) -> float:
        return 1 / self.period

    @property
    def tobs(self) -> float:
        return self.nsamps * self.dt

    @property
    def tol_bins(self) -> float:
        return self.ducy * self.period / self.dt

    @property
    def fold_bins(self) -> int:
        return int(self.period / self.dt / self.ds)

    @property
    def fold_bins_ideal(self) -> int:
        return int(self.period / self.dt)

    @property
    def mod_func(self):
        return self._mod_func

    @property
    def proper_time(self) -> np.ndarray:
        """Proper times of the samples (host, float64)."""
        t = np.arange(self.nsamps, dtype=np.float64) * self.dt
        return self._mod_func.generate(t, self.mod_tref)

    def get_updated(self, update_dict: dict | None) -> PulseSignalConfig:
        names = {f.name for f in fields(self)}
        return replace(self, **{k: v for k, v in (update_dict or {}).items() if k in names})

    def generate(self, shape: str = "gaussian", phi0: float = 0.5, max_iter: int = 5,
                 tol: float = 1e-2, *, seed: int | None = None, noise=None,
                 device=None) -> TimeSeries:
        """A noisy series whose fold at the pulse period has S/N ``snr``
        (device tensors)."""
        b = generate_injections([self], shape, phi0, max_iter, tol, seed=seed,
                                noise=None if noise is None else _rows(noise, 1, self.nsamps),
                                device=device)
        return b.series(0)

    def generate_noise(self, *, seed: int | None = None, device=None) -> TimeSeries:
        """White noise of the standard deviation the configuration implies
        (``pulse.py:225-231``)."""
        std = np.sqrt(self.nsamps * self.ducy) / self.snr / self.tol_bins
        dev = _device(device)
        batch = _Batch([self], "gaussian", 0.5, seed, dev)
        scales = torch.tensor([[std, 0.0, np.nan, np.nan]], dtype=torch.float64, device=dev)
        ts_e, ts_v = batch.emit(scales, None)
        return TimeSeries(ts_e[0], ts_v[0], self.dt)

    def template(self, shape: str = "gaussian", phi0: float = 0.5, *, device=None,
                 return_proper_time: bool = False):
        """The noiseless template (``generate_pulse_template``), float32 on
        the device; with ``return_proper_time`` also the proper times."""
        batch = _Batch([self], shape, phi0, 0, _device(device))
        tm, pt = batch.template(return_proper_time)
        return (tm[0], pt[0]) if return_proper_time else tm[0]


def _rows(x, n: int, nsamps: int) -> torch.Tensor:
    t = torch.as_tensor(x, dtype=torch.float32)
    if t.ndim == 1:
        t = t[None, :]
    if tuple(t.shape) != (n, nsamps):
        msg = f"noise must have shape ({n}, {nsamps}), got {tuple(t.shape)}"
        raise ValueError(msg)
    return t


class _Batch:
    """Device specs, CDF tables and proper-time tables of a set of injections
    with a common length and sampling."""

    def __init__(self, cfgs, shape, phi0, seed, device: torch.device) -> None:
        self.cfgs = list(cfgs)
        if not self.cfgs:
            msg = "no injections"
            raise ValueError(msg)
        n = len(self.cfgs)
        if n > 65535:
            msg = "at most 65535 injections per call"
            raise ValueError(msg)
        self.nsamps = int(self.cfgs[0].nsamps)
        self.device = device
        if any(int(c.nsamps) != self.nsamps for c in self.cfgs):
            msg = "all injections of a batch need the same nsamps"
            raise ValueError(msg)
        shapes = [shape] * n if isinstance(shape, str) else list(shape)
        if len(shapes) != n:
            msg = f"{len(shapes)} shapes for {n} injections"
            raise ValueError(msg)
        phis = np.broadcast_to(np.asarray(phi0, dtype=np.float64), (n,))
        for s in shapes:
            if s not in SHAPES:
                msg = f"Unknown shape: {s}"
                raise ValueError(msg)
        seeds = _seeds(seed, n)
        specs = (_lib.LokiPulseSpec * n)()
        tables = []
        need_table = any(not hasattr(c.mod_func, "encode") for c in self.cfgs)
        self.fold_stride = max(4, max(c.fold_bins_ideal for c in self.cfgs))
        keys = [(s, float(c.ducy), float(ph), max(4096, int(100 / c.ducy)))
                for c, s, ph in zip(self.cfgs, shapes, phis)]
        lut_of = cdf_tables(dict.fromkeys(keys))
        cache: dict = {}
        luts, off = [], 0
        for key in lut_of:
            cache[key] = (off, key[3])
            luts.append(lut_of[key])
            off += key[3] + 1
        for j, (c, key) in enumerate(zip(self.cfgs, keys)):
            ph = key[2]
            sp = specs[j]
            sp.dt, sp.period, sp.snr = float(c.dt), float(c.period), float(c.snr)
            sp.ducy, sp.phi0 = float(c.ducy), float(ph)
            sp.nbins = int(c.fold_bins_ideal)
            sp.lut_off, sp.ngrid = cache[key]
            sp.seed = int(seeds[j])
            if hasattr(c.mod_func, "encode"):
                sp.mod = c.mod_func.encode(c.mod_tref)
            else:
                sp.mod.kind = _lib.MOD_KINDS["table"]
            if need_table:
                tables.append(np.asarray(c.proper_time, dtype=np.float64))
        self.specs = torch.frombuffer(bytearray(bytes(specs)), dtype=torch.uint8).to(device)
        self.luts = torch.from_numpy(np.concatenate(luts)).to(device)
        self.table = (torch.from_numpy(np.stack(tables)).to(device) if need_table else None)
        self.n = n
        self.lib = _lib.load()

    def _stream(self) -> int:
        return _lib.stream_ptr(torch.cuda.current_stream(self.device))

    def template(self, with_pt: bool):
        tm = torch.empty((self.n, self.nsamps), dtype=torch.float32, device=self.device)
        pt = (torch.empty((self.n, self.nsamps), dtype=torch.float64, device=self.device)
              if with_pt else None)
        _lib.check(self.lib.loki_pulse_template(
            _lib.ptr(self.specs), self.n, self.nsamps, _lib.ptr(self.luts),
            _lib.ptr(self.table), _lib.ptr(tm), _lib.ptr(pt), self._stream()))
        return tm, pt

    def fold(self, noise, keep=None) -> torch.Tensor:
        """Calibration folds; ``keep`` = (noise_out, tmpl_out) (n, nsamps)
        float32 receive the unit noise and the template."""
        if self.fold_stride > _lib.PULSE_MAX_NBINS:
            msg = (f"period / dt = {self.fold_stride} calibration bins, above "
                   f"{_lib.PULSE_MAX_NBINS}")
            raise ValueError(msg)
        if min(c.fold_bins_ideal for c in self.cfgs) < 4:
            msg = "period / dt must give at least 4 calibration bins"
            raise ValueError(msg)
        folds = torch.empty((self.n, 3, self.fold_stride), dtype=torch.float64,
                            device=self.device)
        z_out, t_out = keep if keep is not None else (None, None)
        _lib.check(self.lib.loki_pulse_fold(
            _lib.ptr(self.specs), self.n, self.nsamps, _lib.ptr(self.luts),
            _lib.ptr(self.table), _lib.ptr(noise), _lib.ptr(folds), self.fold_stride,
            _lib.ptr(z_out), _lib.ptr(t_out), self._stream()))
        return folds

    def apply(self, scales: torch.Tensor, ts_e: torch.Tensor, ts_v: torch.Tensor) -> None:
        """In place: (noise, template) from ``fold(keep=...)`` become the series."""
        _lib.check(self.lib.loki_pulse_apply(_lib.ptr(scales), self.n, self.nsamps,
                                             _lib.ptr(ts_e), _lib.ptr(ts_v), self._stream()))

    def alloc(self, out=None):
        if out is None:
            ts_e = torch.empty((self.n, self.nsamps), dtype=torch.float32, device=self.device)
            return ts_e, torch.empty_like(ts_e)
        ts_e, ts_v = out
        shape = (self.n, self.nsamps)
        for t in (ts_e, ts_v):
            if (tuple(t.shape) != shape or t.dtype != torch.float32 or not t.is_contiguous()
                    or t.device != self.device):
                msg = f"out tensors must be contiguous float32 {shape} on {self.device}"
                raise ValueError(msg)
        return ts_e, ts_v

    def calibrate(self, folds: torch.Tensor, max_iter: int, tol: float) -> torch.Tensor:
        out = torch.empty((self.n, 4), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.loki_pulse_calibrate(
            _lib.ptr(self.specs), self.n, _lib.ptr(folds), int(folds.shape[-1]), int(max_iter),
            float(tol), _lib.ptr(out), self._stream()))
        return out

    def emit(self, scales: torch.Tensor, noise, out=None):
        """The series regenerated from seeds (or ``noise``) and ``scales``."""
        ts_e, ts_v = self.alloc(out)
        _lib.check(self.lib.loki_pulse_emit(
            _lib.ptr(self.specs), self.n, self.nsamps, _lib.ptr(self.luts),
            _lib.ptr(self.table), _lib.ptr(noise), _lib.ptr(scales), _lib.ptr(ts_e),
            _lib.ptr(ts_v), self._stream()))
        return ts_e, ts_v


@dataclass
class InjectionBatch:
    """Series (n, nsamps) on the device with their calibration:
    ``scales[:, 0]`` noise scale, ``[:, 1]`` signal scale, ``[:, 2]`` S/N of
    the template alone, ``[:, 3]`` last measured S/N."""

    ts_e: torch.Tensor
    ts_v: torch.Tensor
    scales: torch.Tensor
    folds: torch.Tensor
    cfgs: list
    dt: float

    def series(self, i: int) -> TimeSeries:
        return TimeSeries(self.ts_e[i], self.ts_v[i], self.dt)

    def __len__(self) -> int:
        return len(self.cfgs)


def generate_injections(cfgs, shape="gaussian", phi0=0.5, max_iter: int = 5, tol: float = 1e-2,
                        *, seed: int | None = None, noise=None, device=None,
                        out=None) -> InjectionBatch:
    """``PulseSignalConfig.generate`` for every configuration of ``cfgs``
    (same ``nsamps`` and ``dt``) in five kernel launches: the fold pass also
    writes the unit noise and the template into the output arrays, which the
    last pass scales in place. ``shape`` and
    ``phi0`` may be per injection. ``noise`` (n, nsamps) replaces the drawn
    unit noise; ``out`` = (ts_e, ts_v) preallocated (n, nsamps) float32."""
    dev = _device(device)
    cfgs = list(cfgs)
    if any(float(c.dt) != float(cfgs[0].dt) for c in cfgs):
        msg = "all injections of a batch need the same dt"
        raise ValueError(msg)
    batch = _Batch(cfgs, shape, phi0, seed, dev)
    nz = None
    if noise is not None:
        nz = _rows(noise, batch.n, batch.nsamps).to(dev).contiguous()
        if not bool(torch.isfinite(nz).all()) or float(nz.abs().max()) >= 2.0**20:
            msg = "noise must be finite and below 2^20 in magnitude"
            raise ValueError(msg)
    ts_e, ts_v = batch.alloc(out)
    folds = batch.fold(nz, keep=(ts_e, ts_v))
    scales = batch.calibrate(folds, max_iter, tol)
    batch.apply(scales, ts_e, ts_v)
    return InjectionBatch(ts_e, ts_v, scales, folds, cfgs, float(cfgs[0].dt))


def generate_pulse_template(proper_time, dt: float, period: float, cdf_lut,
                            *, device=None) -> torch.Tensor:
    """Template of ``cdf_lut`` over given proper times (float32, device),
    as ``generate_pulse_template``."""
    dev = _device(device)
    lib = _lib.load()
    pt = torch.as_tensor(np.asarray(proper_time, dtype=np.float64)).to(dev).contiguous()
    lut = torch.as_tensor(np.asarray(cdf_lut, dtype=np.float32)).to(dev).contiguous()
    spec = _lib.LokiPulseSpec()
    spec.dt, spec.period = float(dt), float(period)
    spec.ngrid = int(lut.numel()) - 1
    spec.mod.kind = _lib.MOD_KINDS["table"]
    specs = torch.frombuffer(bytearray(bytes(spec)), dtype=torch.uint8).to(dev)
    n = int(pt.numel())
    tm = torch.empty(n, dtype=torch.float32, device=dev)
    _lib.check(lib.loki_pulse_template(
        _lib.ptr(specs), 1, n, _lib.ptr(lut), _lib.ptr(pt), _lib.ptr(tm), 0,
        _lib.stream_ptr(torch.cuda.current_stream(dev))))
    return tm


__all__ = ["InjectionBatch", "PulseSignalConfig", "build_cdf_lut", "generate_injections",
           "generate_pulse_template"]

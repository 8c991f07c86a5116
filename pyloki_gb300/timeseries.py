"""Input series container (``io/timeseries.py:16-40`` TimeSeries)."""

from __future__ import annotations

import numpy as np


def _is_tensor(x) -> bool:
    return type(x).__module__.startswith("torch")


class TimeSeries:
    """A time series as pyloki holds it.

    Parameters
    ----------
    ts_e : array
        Signal weighted by E/V (float32).
    ts_v : array
        Variance term E**2/V (float32), same length as ``ts_e``.
    tsamp : float
        Sampling time in seconds.
    """

    def __init__(self, ts_e, ts_v, tsamp: float) -> None:
        if _is_tensor(ts_e) or _is_tensor(ts_v):
            # torch tensors (pinned host or device memory) are kept as given
            import torch

            ts_e = torch.as_tensor(ts_e).to(dtype=torch.float32).contiguous()
            ts_v = torch.as_tensor(ts_v).to(dtype=torch.float32).contiguous()
        else:
            ts_e = np.asarray(ts_e, dtype=np.float32)
            ts_v = np.asarray(ts_v, dtype=np.float32)
        if ts_e.ndim != 1 or ts_e.shape != ts_v.shape:
            msg = "ts_e and ts_v must be 1-D arrays of the same length"
            raise ValueError(msg)
        if tsamp <= 0:
            msg = f"tsamp must be positive, got {tsamp}"
            raise ValueError(msg)
        self.ts_e = ts_e
        self.ts_v = ts_v
        self.tsamp = float(tsamp)

    @property
    def dt(self) -> float:
        """Sampling time (the reference's name for ``tsamp``)."""
        return self.tsamp

    @property
    def nsamps(self) -> int:
        return len(self.ts_e)

    @property
    def tobs(self) -> float:
        return self.nsamps * self.tsamp

    def pad_to_pow2(self, nsamps: int | None = None) -> TimeSeries:
        """Zero-pad (ts_v = 0 beyond the data) or truncate to a power of two."""
        n = nsamps or 1 << int(np.ceil(np.log2(self.nsamps)))
        e = np.zeros(n, np.float32)
        v = np.zeros(n, np.float32)
        m = min(n, self.nsamps)
        e[:m] = np.asarray(self.ts_e[:m].cpu() if _is_tensor(self.ts_e) else self.ts_e[:m])
        v[:m] = np.asarray(self.ts_v[:m].cpu() if _is_tensor(self.ts_v) else self.ts_v[:m])
        return TimeSeries(e, v, self.tsamp)

    def _device_arrays(self, device):
        import torch

        dev = torch.device(device) if device is not None else (
            self.ts_e.device if _is_tensor(self.ts_e) and self.ts_e.is_cuda
            else torch.device("cuda", torch.cuda.current_device()))
        host = not (_is_tensor(self.ts_e) and self.ts_e.is_cuda)
        e = torch.as_tensor(self.ts_e).to(dev, torch.float32).contiguous()
        v = torch.as_tensor(self.ts_v).to(dev, torch.float32).contiguous()
        return e, v, dev, host

    def downsample(self, factor: int, *, device=None) -> TimeSeries:
        """Means of ``factor`` consecutive samples (``io/timeseries.py:40-43``,
        ``np_utils.downsample_1d``), on the GPU. As in the reference the new
        series keeps this series' sampling time."""
        import torch

        from pyloki_gb300 import _lib

        e, v, dev, host = self._device_arrays(device)
        n = self.nsamps // int(factor)
        out = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(2)]
        stream = _lib.stream_ptr(torch.cuda.current_stream(dev))
        for src, dst in zip((e, v), out):
            _lib.check(_lib.load().loki_downsample(_lib.ptr(src), src.numel(), int(factor),
                                                   _lib.ptr(dst), stream))
        if host:
            out = [t.cpu().numpy() for t in out]
        return TimeSeries(out[0], out[1], self.tsamp)

    def fold_ephem(self, freq: float, nbins: int, nsubints: int = 1, *, normalize: bool = True,
                   mod_type: str = "derivative", mod_kwargs: dict | None = None,
                   mod_tref: float | None = None, device=None):
        """The series folded at ``freq`` over the proper times of a modulation
        model (``io/timeseries.py:45-83``): ``(2, nbins)`` or
        ``(nsubints, 2, nbins)`` sums, or with ``normalize`` the profiles
        e / sqrt(v) (0 where the variance is within 1e-5 of zero). The sums
        are the reference's bit for bit (GPU, sample order)."""
        import torch

        from pyloki_gb300 import _lib
        from pyloki_gb300.modulate import type_to_mods

        cycles = int(self.tobs * freq)
        if cycles < 1:
            msg = f"Period ({1 / freq}) is less than the total data length ({self.tobs})"
            raise ValueError(msg)
        if nsubints < 1 or nsubints > cycles:
            msg = f"subints must be >= 1 and <= {cycles}"
            raise ValueError(msg)
        mod_tref = self.tobs / 2 if mod_tref is None else mod_tref
        mod_func = type_to_mods[mod_type](**(mod_kwargs or {}))
        e, v, dev, host = self._device_arrays(device)
        table = None
        if hasattr(mod_func, "encode"):
            mod = mod_func.encode(mod_tref)
        else:
            mod = _lib.LokiModulation()
            mod.kind = _lib.MOD_KINDS["table"]
            t = np.arange(self.nsamps, dtype=np.float64) * self.tsamp
            table = torch.from_numpy(np.asarray(mod_func.generate(t, mod_tref),
                                                dtype=np.float64)).to(dev)
        bins = torch.empty(self.nsamps, dtype=torch.int32, device=dev)
        fold = torch.empty((nsubints, 2, nbins), dtype=torch.float32, device=dev)
        norm = torch.empty((nsubints, nbins), dtype=torch.float32, device=dev) if normalize \
            else None
        _lib.check(_lib.load().loki_fold_ephem(
            _lib.ptr(e), _lib.ptr(v), self.nsamps, self.tsamp, mod, _lib.ptr(table),
            float(freq), int(nbins), int(nsubints), _lib.ptr(bins), _lib.ptr(fold),
            _lib.ptr(norm), _lib.stream_ptr(torch.cuda.current_stream(dev))))
        res = (norm if normalize else fold).squeeze(0) if nsubints == 1 else (
            norm if normalize else fold)
        return res.cpu().numpy() if host else res

    def __str__(self) -> str:
        return (f"{type(self).__name__} {{nsamps = {self.nsamps:d}, tsamp = {self.tsamp:.4e}, "
                f"tobs = {self.tobs:.3f}}}")

    __repr__ = __str__

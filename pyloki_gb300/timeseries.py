"""Input series container (``io/timeseries.py:16-40`` TimeSeries)."""

from __future__ import annotations

import numpy as np


def _is_tensor(x) -> bool:
    return type(x).__module__.startswith("torch")


class _Stats:
    """Order statistics, sums and moments of one device array (float32),
    each computed by the library's kernels and read back as a float."""

    def __init__(self, x, dev) -> None:
        import torch

        from pyloki_gb300 import _lib

        self.x, self.dev, self.n = x, dev, int(x.numel())
        if self.n < 1:
            msg = "statistics of an empty series"
            raise ValueError(msg)
        self.lib = _lib.load()
        self.stream = _lib.stream_ptr(torch.cuda.current_stream(dev))
        self._scratch = torch.empty(max(int(self.lib.loki_select_scratch_bytes()), 8192),
                                    dtype=torch.uint8, device=dev)
        self._val = torch.empty(1, dtype=torch.float32, device=dev)
        self._dval = torch.empty(1, dtype=torch.float64, device=dev)

    def kth(self, k: int, x=None) -> float:
        from pyloki_gb300 import _lib

        x = self.x if x is None else x
        _lib.check(self.lib.loki_select_kth(_lib.ptr(x), x.numel(), int(k), _lib.ptr(self._val),
                                            _lib.ptr(self._scratch), self._scratch.numel(),
                                            self.stream))
        return float(self._val.item())

    def _sum(self, x, square: bool) -> float:
        from pyloki_gb300 import _lib

        _lib.check(self.lib.loki_sum_f64(_lib.ptr(x), x.numel(), int(square),
                                         _lib.ptr(self._dval), _lib.ptr(self._scratch),
                                         self._scratch.numel(), self.stream))
        return float(self._dval.item())

    def mean(self) -> float:
        return self._sum(self.x, False) / self.n

    def median(self, x=None) -> float:
        n = self.n if x is None else int(x.numel())
        lo = self.kth((n - 1) // 2, x)
        hi = lo if n % 2 else self.kth(n // 2, x)
        return float(np.float32((np.float64(lo) + np.float64(hi)) / 2.0))

    def percentile(self, q: float) -> float:
        """numpy's ``percentile`` (linear interpolation) of the array."""
        pos = (self.n - 1) * q / 100.0
        k = int(np.floor(pos))
        t = pos - k
        a = np.float64(self.kth(k))
        b = np.float64(self.kth(min(k + 1, self.n - 1))) if t > 0 else a
        return float(a + (b - a) * t) if t < 0.5 else float(b - (b - a) * (1.0 - t))

    def _dev(self, loc: float, absolute: bool):
        import torch

        from pyloki_gb300 import _lib

        d = torch.empty_like(self.x)
        _lib.check(self.lib.loki_affine(_lib.ptr(self.x), self.n, float(np.float32(loc)),
                                        0.0 if absolute else 1.0, _lib.ptr(d), self.stream))
        return d

    def std(self) -> float:
        return float(np.sqrt(self._sum(self._dev(self.mean(), False), True) / self.n))

    def mad(self) -> float:
        return self.median(self._dev(self.median(), True))


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

    def deredden(self, method: str = "median", window: float = 0.5, *, fast: bool = False,
                 device=None) -> TimeSeries:
        """``ts_e`` minus its running median over ``window`` seconds
        (``int(window / tsamp)`` samples, as the reference's call into
        sigpyproc's ``TimeSeries.deredden``, ``io/timeseries.py:231``), on the
        GPU: the order statistic of rank ``window // 2`` of the centred window
        with half-sample symmetric reflection at the ends (the definition of
        ``scipy.ndimage.median_filter``, mode ``"reflect"``). ``fast`` is
        accepted for the reference's signature; the filter is always exact.
        ``ts_v`` is kept."""
        import torch

        from pyloki_gb300 import _lib

        del fast
        if method != "median":
            msg = f"deredden method must be 'median', got {method!r}"
            raise ValueError(msg)
        nwin = int(window / self.tsamp)
        if nwin < 1:
            msg = f"window {window} s is shorter than one sample ({self.tsamp} s)"
            raise ValueError(msg)
        e, v, dev, host = self._device_arrays(device)
        if not bool(torch.isfinite(e).all()):
            msg = "deredden needs a finite series (no NaN or inf)"
            raise ValueError(msg)
        out = torch.empty_like(e)
        _lib.check(_lib.load().loki_running_median(
            _lib.ptr(e), e.numel(), nwin, 1, _lib.ptr(out),
            _lib.stream_ptr(torch.cuda.current_stream(dev))))
        return TimeSeries(out.cpu().numpy() if host else out,
                          v.cpu().numpy() if host else v, self.tsamp)

    def normalise(self, loc_method: str = "mean", scale_method: str = "std", *,
                  device=None) -> TimeSeries:
        """``(ts_e - loc) / scale`` in float32 (the reference's call into
        sigpyproc's ``TimeSeries.normalise``, ``io/timeseries.py:232``), with
        the statistics taken on the GPU:

        - ``loc_method``: ``"mean"`` (float64 sum / n) or ``"median"`` (the
          mean of the two middle order statistics for an even count);
        - ``scale_method``: ``"std"`` (population standard deviation about
          the mean, float64), ``"iqr"`` (interquartile range of numpy's
          linearly interpolated percentiles / 1.3489795003921634, the normal
          consistency factor) or ``"mad"`` (median absolute deviation about
          the median x 1.482602218505602).

        ``ts_v`` is kept."""
        import torch

        from pyloki_gb300 import _lib

        e, v, dev, host = self._device_arrays(device)
        st = _Stats(e, dev)
        if loc_method == "mean":
            loc = st.mean()
        elif loc_method == "median":
            loc = st.median()
        else:
            msg = f"loc_method must be 'mean' or 'median', got {loc_method!r}"
            raise ValueError(msg)
        if scale_method == "std":
            scale = st.std()
        elif scale_method == "iqr":
            scale = (st.percentile(75.0) - st.percentile(25.0)) / 1.3489795003921634
        elif scale_method == "mad":
            scale = st.mad() * 1.482602218505602
        else:
            msg = f"scale_method must be 'std', 'iqr' or 'mad', got {scale_method!r}"
            raise ValueError(msg)
        if not scale > 0 or not np.isfinite(scale):
            msg = f"the series has scale {scale}: it cannot be normalised"
            raise ValueError(msg)
        out = torch.empty_like(e)
        _lib.check(_lib.load().loki_affine(_lib.ptr(e), e.numel(), float(np.float32(loc)),
                                           float(np.float32(scale)), _lib.ptr(out),
                                           st.stream))
        return TimeSeries(out.cpu().numpy() if host else out,
                          v.cpu().numpy() if host else v, self.tsamp)

    @classmethod
    def from_tim(cls, timfile, tim_type: str = "dat", filter_window: float = 1.0,
                 norm_scale_method: str = "iqr", *, device=None) -> TimeSeries:
        """Load a ``.dat`` (PRESTO, with its ``.inf``) or ``.tim`` (SIGPROC)
        series, deredden it with a running median of ``filter_window``
        seconds, normalise it to zero mean and unit ``norm_scale_method``
        scale, and pair it with unit variance
        (``io/timeseries.py:198-236``). The filters run on the GPU."""
        from pyloki_gb300 import sigproc

        if tim_type == "dat":
            data, info = sigproc.read_dat(timfile)
            tsamp = info["tsamp"]
        elif tim_type == "tim":
            data, hdr = sigproc.read_tim(timfile)
            tsamp = hdr["tsamp"]
        else:
            msg = f"Invalid tim type: {tim_type}"
            raise ValueError(msg)
        ts = cls(data, np.ones_like(data), tsamp)
        ts = ts.deredden(method="median", window=filter_window, fast=True, device=device)
        ts = ts.normalise(loc_method="mean", scale_method=norm_scale_method, device=device)
        return cls(ts.ts_e, np.ones_like(ts.ts_e) if not _is_tensor(ts.ts_e)
                   else ts.ts_e.new_ones(ts.ts_e.shape), tsamp)

    def __str__(self) -> str:
        return (f"{type(self).__name__} {{nsamps = {self.nsamps:d}, tsamp = {self.tsamp:.4e}, "
                f"tobs = {self.tobs:.3f}}}")

    __repr__ = __str__

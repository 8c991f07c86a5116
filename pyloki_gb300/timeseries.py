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

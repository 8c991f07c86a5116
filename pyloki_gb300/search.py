"""Top-level FFA period search (``search.py:17-53``) and its periodogram.

``ffa_search`` returns ``(DynamicProgramming, Periodogram)`` like the
reference. The S/N array stays on the device; ``Periodogram`` offers the
reference's ``find_best_indices`` / ``find_best_params`` / ``get_summary``
(``periodogram.py:25-200``) without the xarray/plotting layer.
"""

from __future__ import annotations

import numpy as np
import torch

from pyloki_gb300.config import PulsarSearchConfig
from pyloki_gb300.ffa import DynamicProgramming
from pyloki_gb300.timeseries import TimeSeries


class Periodogram:
    """S/N over (*params, width) with the reference's accessors."""

    REQUIRED_PARAMS = ("freq", "width")
    OPTIONAL_PARAMS = ("crackle", "snap", "jerk", "accel")

    def __init__(self, params: dict[str, np.ndarray], snrs, tobs: float) -> None:
        self.params = params
        self.snrs = snrs
        self.tobs = float(tobs)
        shape = tuple(len(params[p]) for p in self.param_names)
        if tuple(snrs.shape) != shape:
            msg = f"snrs shape {tuple(snrs.shape)} does not match params {shape}"
            raise ValueError(msg)

    @property
    def param_names(self) -> list[str]:
        return [p for p in self.OPTIONAL_PARAMS + self.REQUIRED_PARAMS if p in self.params]

    @property
    def ndim(self) -> int:
        return len(self.param_names)

    def find_best_indices(self, *, ignore_nan: bool = False) -> tuple[int, ...]:
        """Index of the maximum S/N. Like the reference (``np.argmax``) a NaN
        S/N (a profile with an empty bin: e / sqrt(0)) wins unless
        ``ignore_nan`` is set."""
        if isinstance(self.snrs, torch.Tensor):
            s = torch.nan_to_num(self.snrs, nan=-torch.inf) if ignore_nan else self.snrs
            flat = int(torch.argmax(s).item())
        else:
            s = np.where(np.isnan(self.snrs), -np.inf, self.snrs) if ignore_nan else self.snrs
            flat = int(np.argmax(s))
        return tuple(int(i) for i in np.unravel_index(flat, tuple(self.snrs.shape)))

    def find_best_params(self, *, ignore_nan: bool = False) -> dict[str, float]:
        idx = self.find_best_indices(ignore_nan=ignore_nan)
        best = {name: self.params[name][i] for name, i in zip(self.param_names, idx, strict=False)}
        return {"snr": float(self.snrs[idx]), **best}

    def get_summary(self) -> str:
        best = self.find_best_params()
        lines = [f"Best S/N: {best['snr']:.2f}", f"Best Period: {1 / best['freq']}"]
        lines += [f"Best {name}: {best[name]}" for name in self.param_names]
        return "\n".join(lines)

    def __repr__(self) -> str:
        info = ", ".join(f"{p}: {len(self.params[p])}" for p in self.param_names)
        return f"Periodogram({info}, tobs: {self.tobs})"


def ffa_search(tseries: TimeSeries, search_cfg: PulsarSearchConfig, *, quiet: bool = False,
               show_progress: bool = False, materialize: bool | None = None,
               device=None, norm: str = "exact") -> tuple[DynamicProgramming, Periodogram]:
    """FFA search: brute fold, DP levels, boxcar S/N of segment 0.

    With ``materialize`` (default: when the final fold is at most 1 GiB) every
    level is kept, as in the reference, and ``dyp.fold`` is the final fold;
    otherwise the last levels are fused with scoring (``dyp.search``) and only
    the S/N array is produced. Both paths give identical S/N. ``norm="fast"``
    (fused path only) normalises profiles with the reciprocal square root:
    S/N within 1e-5 of the reference relative to max(|S/N|, 1).
    """
    dyp = DynamicProgramming(tseries, search_cfg, device=device)
    widths = search_cfg.score_widths
    if materialize is None:
        materialize = dyp.level_bytes(search_cfg.niters_ffa) <= 1 << 30
    dyp.initialize()
    if materialize:
        dyp.execute(show_progress=show_progress)
        from pyloki_gb300.scoring import boxcar_snr_nd

        snrs = boxcar_snr_nd(dyp.get_fold_norm(), widths, 1.0)
    else:
        snrs = dyp.search(widths, 1.0, norm=norm)
    pgram = Periodogram(params={"width": widths, **dyp.param_arr_dict}, snrs=snrs,
                        tobs=tseries.tobs)
    return dyp, pgram

"""Top-level FFA period search (``search.py:17-53``) and its periodogram.

``ffa_search`` returns ``(DynamicProgramming, Periodogram)`` like the
reference. The S/N array stays on the device; ``Periodogram`` offers the
reference's ``find_best_indices`` / ``find_best_params`` / ``get_summary``
(``periodogram.py:25-200``) and ``save`` / ``load`` in xarray's NetCDF
layout, without the xarray/plotting layer.
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

    #: the variable name xarray gives an unnamed DataArray in a file
    DATA_VAR = "__xarray_dataarray_variable__"

    def save(self, filename) -> None:
        """The periodogram as xarray's ``DataArray.to_netcdf`` writes it
        (``periodogram.py:165-166``) when no netCDF-4 library is present:
        a NetCDF-3 (64-bit offset) file with one coordinate variable per
        parameter and the S/N variable carrying ``tobs``. Integer
        coordinates are stored as int32, as xarray coerces them for
        NetCDF-3."""
        from scipy.io import netcdf_file

        snrs = self.snrs.cpu().numpy() if isinstance(self.snrs, torch.Tensor) else self.snrs
        with netcdf_file(filename, "w", version=2) as f:
            for name in self.param_names:
                vals = np.asarray(self.params[name])
                if vals.dtype.kind in "iu":
                    vals = vals.astype(np.int32)
                else:
                    vals = vals.astype(np.float64)
                f.createDimension(name, len(vals))
                var = f.createVariable(name, vals.dtype, (name,))
                var[:] = vals
            data = np.ascontiguousarray(snrs, np.float32)
            var = f.createVariable(self.DATA_VAR, data.dtype, tuple(self.param_names))
            var[...] = data
            var.tobs = np.float64(self.tobs)  # NC_DOUBLE (a Python float would be NC_FLOAT)

    @classmethod
    def load(cls, filename) -> Periodogram:
        """A periodogram written by ``save`` or by the reference with
        xarray's NetCDF-3 backend (``periodogram.py:168-172``)."""
        from scipy.io import netcdf_file

        with open(filename, "rb") as fh:
            if fh.read(3) != b"CDF":
                msg = f"{filename}: not a NetCDF-3 file (NetCDF-4 files need a netCDF-4 reader)"
                raise ValueError(msg)
        with netcdf_file(filename, "r", mmap=False) as f:
            data_vars = [k for k, v in f.variables.items()
                         if not (v.dimensions == (k,))]
            if len(data_vars) != 1:
                msg = f"{filename}: expected one data variable, found {data_vars}"
                raise ValueError(msg)
            var = f.variables[data_vars[0]]
            params = {}
            for dim in var.dimensions:
                vals = np.array(f.variables[dim][:])
                params[dim] = vals.astype(np.int64) if vals.dtype.kind in "iu" else vals
            snrs = np.array(var[...])
            tobs = float(var.tobs)
        return cls(params=params, snrs=snrs, tobs=tobs)


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

"""Search configuration and grid arithmetic (host side, FP64).

Mirrors pyloki's ``PulsarSearchConfig`` / ``ParamLimits`` (``config.py:59-827``)
and the grid helpers they call (``utils/psr_utils.py:59-143,401-463``,
``detection/scoring.py:10-39``, ``utils/maths.py:11-34``). Every expression
keeps the reference's numpy operation order so the grids (and therefore the
integer plan tables computed from them on the GPU) are bit-identical.

The class is a frozen dataclass rather than an ``attrs`` class so that it
imports on machines without ``attrs``; field names, defaults, validation
rules and error types are the reference's.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

#: Speed of light (m/s), the value pyloki takes from astropy (``utils/misc.py:38``).
C_VAL = 299792458.0
#: Rounding guard used by every grid-index truncation (``utils/misc.py:40``).
FLOAT_EPSILON = 1e-6

_FACT_TAB = np.array([float(math.factorial(i)) for i in range(120)], dtype=np.float64)


def fact(num):
    """Factorial as float64, table-driven like ``utils/maths.py:11-34``."""
    num = np.asarray(num)
    out = _FACT_TAB[np.clip(num, 0, 119)]
    return out if out.ndim else float(out)


def is_power_of_two(n: int) -> bool:
    return n > 0 and (n & (n - 1)) == 0


def generate_box_width_trials(nbins: int, ducy_max: float = 0.2,
                              wtsp: float = 1.5) -> np.ndarray:
    """Boxcar width trials (``detection/scoring.py:10-39``)."""
    wmax = int(max(1, ducy_max * nbins))
    widths = [1]
    while widths[-1] <= wmax:
        next_width = int(max(widths[-1] + 1, int(wtsp * widths[-1])))
        if next_width > wmax:
            break
        widths.append(next_width)
    return np.asarray(widths, dtype=np.int64)


def poly_taylor_step_f(nparams: int, tobs: float, nbins: int, eta: float,
                       t_ref: float = 0, use_cheby: bool = True) -> np.ndarray:
    """Grid step for {f_k, ..., f_0} (``utils/psr_utils.py:59-95``)."""
    dphi = eta / nbins
    k = np.arange(nparams)
    dparams_f = dphi * fact(k + 1) / (tobs - t_ref) ** (k + 1)
    if use_cheby:
        dparams_f = 2**k * dparams_f
    return dparams_f[::-1]


def poly_taylor_step_d_f(nparams: int, tobs: float, nbins: int, eta: float,
                         f_max: float, t_ref: float = 0,
                         use_cheby: bool = True) -> np.ndarray:
    """Grid step for {d_k, ..., d_2, f} (``utils/psr_utils.py:98-113``)."""
    dparams_f = poly_taylor_step_f(nparams, tobs, nbins, eta, t_ref, use_cheby)
    dparams = np.zeros(nparams, dtype=np.float64)
    dparams[:-1] = dparams_f[:-1] * C_VAL / f_max
    dparams[-1] = dparams_f[-1]
    return dparams


def range_param_count(vmin: float, vmax: float, dv: float) -> int:
    """Number of cell centres (``utils/psr_utils.py:401-424``)."""
    if not (vmin < vmax and dv > 0.0):
        msg = "Invalid input: ensure vmin < vmax and dv > 0.0."
        raise ValueError(msg)
    if dv >= (vmax - vmin):
        return 1
    return math.ceil((vmax - vmin) / dv)


def range_param(vmin: float, vmax: float, dv: float) -> np.ndarray:
    """Cell centres tiling [vmin, vmax] (``utils/psr_utils.py:427-463``)."""
    if not (vmin < vmax and dv > 0):
        msg = "Invalid input: ensure vmin < vmax and dv > 0."
        raise ValueError(msg)
    if dv >= (vmax - vmin):
        return np.array([(vmax + vmin) / 2.0])
    npoints = math.ceil((vmax - vmin) / dv)
    dv_actual = (vmax - vmin) / npoints
    return np.linspace(vmin + (dv_actual / 2.0), vmax - (dv_actual / 2.0), npoints)


def shift_taylor_params(taylor_param_vec: np.ndarray, delta_t: float) -> np.ndarray:
    """Taylor re-referencing by the lower-triangular shift matrix
    (``utils/transforms.py:10-48``); used by the limit factories only."""
    n_params = taylor_param_vec.shape[-1]
    powers = np.tril(np.arange(n_params)[:, np.newaxis] - np.arange(n_params))
    t_mat = delta_t**powers / fact(powers) * np.tril(np.ones_like(powers))
    return np.ascontiguousarray(taylor_param_vec) @ t_mat.T


class ParamLimits:
    """Search parameter bounds, order [..., jerk, accel, freq] (``config.py:59-321``)."""

    def __init__(self, limits) -> None:
        self.limits = np.asarray(limits, dtype=np.float64)

    @classmethod
    def from_taylor(cls, freq, accel=None, jerk=None, snap=None) -> ParamLimits:
        default_limit = (0.0, 0.0)
        all_params = [snap, jerk, accel, freq]
        last_non_none = next(i for i, p in enumerate(all_params) if p is not None)
        out = [p if p is not None else default_limit for p in all_params[last_non_none:]]
        return cls([(float(lo), float(hi)) for lo, hi in out])

    @classmethod
    def from_upper(cls, freq, true_d_params, d_upper_limits, t_obs) -> ParamLimits:
        nparams = len(true_d_params) + 1
        dvec = np.zeros(nparams + 1, dtype=np.float64)
        dvec[1:-2] = true_d_params[1:]
        dvec[0] = d_upper_limits[0]
        dvec_min_up = shift_taylor_params(dvec, t_obs / 2)
        dvec_min_low = shift_taylor_params(dvec, -t_obs / 2)
        dvec[0] = d_upper_limits[1]
        dvec_max_up = shift_taylor_params(dvec, t_obs / 2)
        dvec_max_low = shift_taylor_params(dvec, -t_obs / 2)
        low = np.minimum(dvec_min_low, dvec_max_low)
        up = np.maximum(dvec_min_up, dvec_max_up)
        bounds = list(zip(low, up, strict=False))[:-2]
        freq_shift = up[-2] / C_VAL
        if isinstance(freq, (tuple, list, np.ndarray)):
            fmin, fmax = freq
            bounds.append((fmin * (1 - freq_shift), fmax * (1 + freq_shift)))
        else:
            bounds.append((freq * (1 - freq_shift), freq * (1 + freq_shift)))
        return cls(bounds)

    @classmethod
    def from_circular(cls, freq, p_orb_min: float, m_c_max: float = 10.0,
                      m_p_min: float = 1.2, poly_order: int = 5) -> ParamLimits:
        poly_order = max(poly_order, 2)
        omega_orb_max = 2 * np.pi / p_orb_min
        x_const = float((1.988409870698051e30 * 6.6743e-11) ** (1 / 3)
                        / (C_VAL * (2 * np.pi) ** (2 / 3)))
        x_orb = (x_const * ((m_p_min + m_c_max) * p_orb_min**2) ** (1 / 3)
                 * m_c_max / (m_p_min + m_c_max))
        max_derivs = x_orb * C_VAL * omega_orb_max ** np.arange(poly_order + 1)
        bounds = [(-d, d) for d in max_derivs[2:][::-1]]
        freq_shift = max_derivs[1] / C_VAL
        if isinstance(freq, (tuple, list, np.ndarray)):
            fmin, fmax = freq
            bounds.append((fmin * (1 - freq_shift), fmax * (1 + freq_shift)))
        else:
            bounds.append((freq * (1 - freq_shift), freq * (1 + freq_shift)))
        return cls(bounds)


def _check_limits(value: np.ndarray) -> None:
    if value.shape[0] < 1:
        msg = f"param_limits must have 1-5 elements, got {value.shape[0]}"
        raise ValueError(msg)
    for i in range(value.shape[0]):
        if value[i, 0] >= value[i, 1]:
            msg = f"param_limits must have min < max, got {value}"
            raise ValueError(msg)


@dataclasses.dataclass(frozen=True, kw_only=True)
class PulsarSearchConfig:
    """Configuration of the FFA + pruning search (``config.py:324-827``)."""

    nsamps: int
    tsamp: float
    nbins: int
    eta: float
    param_limits: np.ndarray
    ducy_max: float = 0.2
    wtsp: float = 1.5
    prune_poly_order: int = 3
    p_orb_min: float = 0
    m_c_max: float = 10.0
    m_p_min: float = 1.4
    bseg_brute: int = 0
    bseg_ffa: int = 0
    use_fourier: bool = True
    branch_max: int = 16
    propagator_significance: float = 2.0
    validation_significance: float = 5.0
    tiling_strategy: str = "aggressive"

    def __post_init__(self) -> None:
        limits = np.asarray(self.param_limits, dtype=np.float64)
        if limits.ndim != 2 or limits.shape[1] != 2:
            msg = f"param_limits must be tuples of numbers, got {limits}"
            raise TypeError(msg)
        _check_limits(limits)
        object.__setattr__(self, "param_limits", limits)
        for name in ("nsamps", "nbins", "prune_poly_order", "bseg_brute",
                     "bseg_ffa", "branch_max"):
            if not isinstance(getattr(self, name), (int, np.integer)):
                msg = f"'{name}' must be an int"
                raise TypeError(msg)
        if self.nsamps <= 0 or not is_power_of_two(int(self.nsamps)):
            msg = f"'nsamps' must be a power of 2: {self.nsamps}"
            raise ValueError(msg)
        for name in ("tsamp", "eta", "ducy_max", "wtsp", "propagator_significance",
                     "validation_significance"):
            if not getattr(self, name) > 0:
                msg = f"'{name}' must be > 0"
                raise ValueError(msg)
        if self.nbins <= 0:
            msg = "'nbins' must be > 0"
            raise ValueError(msg)
        if self.prune_poly_order <= 1:
            msg = "'prune_poly_order' must be > 1"
            raise ValueError(msg)
        if self.branch_max <= 10:
            msg = "'branch_max' must be > 10"
            raise ValueError(msg)
        if self.tiling_strategy not in ("aggressive", "quadrature", "conservative"):
            msg = f"'tiling_strategy' must be in aggressive/quadrature/conservative"
            raise ValueError(msg)
        for name in ("bseg_brute", "bseg_ffa"):
            v = int(getattr(self, name))
            if v != 0 and not is_power_of_two(v):
                msg = f"'{name}' must be a power of 2: {v}"
                raise ValueError(msg)
        if self.bseg_brute == 0:
            object.__setattr__(self, "bseg_brute", self._bseg_brute_default())
        if self.bseg_ffa == 0:
            object.__setattr__(self, "bseg_ffa", self._bseg_ffa_default())
        if self.bseg_brute > self.nsamps:
            msg = f"bseg_brute ({self.bseg_brute}) must be < nsamps ({self.nsamps})"
            raise ValueError(msg)
        if self.bseg_ffa > self.nsamps:
            msg = f"bseg_ffa ({self.bseg_ffa}) must be <= nsamps ({self.nsamps})"
            raise ValueError(msg)
        if self.bseg_ffa <= self.bseg_brute:
            msg = f"bseg_ffa ({self.bseg_ffa}) must be > bseg_brute ({self.bseg_brute})"
            raise ValueError(msg)
        if self.prune_poly_order == 5 and self.p_orb_min == 0:
            msg = "p_orb_min must be provided for a circular orbit search"
            raise ValueError(msg)

    # ---- derived quantities (config.py:438-490) ----
    @property
    def tseg_brute(self) -> float:
        return self.bseg_brute * self.tsamp

    @property
    def tseg_ffa(self) -> float:
        return self.bseg_ffa * self.tsamp

    @property
    def niters_ffa(self) -> int:
        return int(np.log2(self.bseg_ffa / self.bseg_brute))

    @property
    def nparams(self) -> int:
        return self.param_limits.shape[0]

    @property
    def param_names(self) -> list[str]:
        return ["crackle", "snap", "jerk", "accel", "freq"][-self.nparams:]

    @property
    def f_min(self) -> float:
        return self.param_limits[-1][0]

    @property
    def f_max(self) -> float:
        return self.param_limits[-1][1]

    @property
    def x_mass_const(self) -> float:
        k_const = float((1.988409870698051e30 * 6.6743e-11) ** (1 / 3))
        return k_const * 1.1 * self.m_c_max / (self.m_p_min + self.m_c_max) ** (2 / 3)

    @property
    def score_widths(self) -> np.ndarray:
        return generate_box_width_trials(self.nbins, ducy_max=self.ducy_max,
                                         wtsp=self.wtsp)

    # ---- per-level grids (config.py:492-634) ----
    def get_dparams_f(self, ffa_level: int) -> np.ndarray:
        tseg_cur = 2**ffa_level * self.tseg_brute
        t_ref = 0 if self.nparams == 1 else tseg_cur / 2
        return poly_taylor_step_f(self.nparams, tseg_cur, self.nbins, self.eta,
                                  t_ref=t_ref)

    def get_dparams(self, ffa_level: int, use_cheby_coarsening: bool = True) -> np.ndarray:
        tseg_cur = 2**ffa_level * self.tseg_brute
        t_ref = 0 if self.nparams == 1 else tseg_cur / 2
        return poly_taylor_step_d_f(self.nparams, tseg_cur, self.nbins, self.eta,
                                    self.f_max, t_ref=t_ref,
                                    use_cheby=use_cheby_coarsening)

    def get_dparams_actual(self, ffa_level: int,
                           use_cheby_coarsening: bool = True) -> np.ndarray:
        counts = self.get_param_grid_count(ffa_level, use_cheby_coarsening)
        out = np.zeros(self.nparams, dtype=np.float64)
        for i in range(self.nparams):
            vmin, vmax = self.param_limits[i]
            out[i] = (vmax - vmin) / counts[i]
        return out

    def get_param_grid_count(self, ffa_level: int,
                             use_cheby_coarsening: bool = True) -> np.ndarray:
        dparams = self.get_dparams(ffa_level, use_cheby_coarsening)
        count = np.empty(self.nparams, dtype=np.int64)
        for i in range(self.nparams):
            count[i] = range_param_count(self.param_limits[i, 0],
                                         self.param_limits[i, 1], dparams[i])
        return count

    def get_param_arr(self, dparams: np.ndarray) -> list[np.ndarray]:
        if len(dparams) != self.nparams:
            msg = f"dparams must have length {self.nparams}, got {len(dparams)}"
            raise ValueError(msg)
        return [range_param(self.param_limits[i, 0], self.param_limits[i, 1],
                            dparams[i]) for i in range(self.nparams)]

    def _bseg_brute_default(self) -> int:
        init_levels = 1 if self.nparams == 1 else 5
        levels = int(np.log2(self.nsamps * self.tsamp * self.f_min) - init_levels)
        return int(self.nsamps / 2**levels)

    def _bseg_ffa_default(self) -> int:
        return self.nsamps

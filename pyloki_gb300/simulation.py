"""Seeded synthetic pulsar series for tests and benchmarks.

The model follows pyloki's generator (``simulation/pulse.py:38-71,500-509``,
``simulation/modulate.py:23-213``): white Gaussian noise plus a von Mises
pulse whose arrival phase is modulated by a line-of-sight Taylor polynomial
(acceleration, jerk) or a circular orbit. Unlike the reference (which draws
from an unseeded generator) every draw here comes from a seeded PCG64, and
the amplitude is set analytically from the target matched-filter S/N
(S/N = A * sqrt(sum(template**2)) for unit-variance noise).
"""

from __future__ import annotations

import numpy as np

from pyloki_gb300.config import C_VAL
from pyloki_gb300.timeseries import TimeSeries


def von_mises_kappa(ducy: float) -> float:
    """Concentration giving a full width at half maximum of ``ducy`` turns."""
    return np.log(2.0) / (2.0 * np.sin(np.pi * ducy / 2.0) ** 2)


def los_delay(t: np.ndarray, t_c: float, accel: float = 0.0, jerk: float = 0.0) -> np.ndarray:
    """Light-travel delay (s) of a Taylor line-of-sight motion about ``t_c``."""
    dt = t - t_c
    return (accel * dt**2 / 2 + jerk * dt**3 / 6) / C_VAL


def circular_delay(t: np.ndarray, p_orb: float, x_orb: float, psi: float) -> np.ndarray:
    """Roemer delay (s) of a circular orbit with projected radius ``x_orb`` (lt-s)."""
    return x_orb * np.sin(2 * np.pi * t / p_orb + psi)


def make_series(nsamps: int, tsamp: float, *, freq: float | None = None, snr: float = 0.0,
                ducy: float = 0.05, accel: float = 0.0, jerk: float = 0.0,
                orbit: tuple[float, float, float] | None = None, phi0: float = 0.5,
                seed: int = 0) -> TimeSeries:
    """Noise N(0, 1) plus an optional pulse at frequency ``freq`` (Hz) and S/N."""
    rng = np.random.default_rng(seed)
    ts_e = rng.standard_normal(nsamps, dtype=np.float32)
    ts_v = np.ones(nsamps, dtype=np.float32)
    if freq is not None and snr > 0:
        t = np.arange(nsamps, dtype=np.float64) * tsamp
        t_c = nsamps * tsamp / 2
        delay = los_delay(t, t_c, accel, jerk)
        if orbit is not None:
            delay = delay + circular_delay(t, *orbit)
        phase = (t - delay) * freq
        kappa = von_mises_kappa(ducy)
        tmpl = np.exp(kappa * (np.cos(2 * np.pi * (phase - phi0)) - 1.0))
        amp = snr / np.sqrt(np.sum(tmpl**2))
        ts_e = (ts_e + amp * tmpl).astype(np.float32)
    return TimeSeries(ts_e, ts_v, tsamp)

"""Time-modulation models of the synthetic pulsar generator
(``simulation/modulate.py``): each maps barycentric times to proper times.

Every model has the reference's ``generate(t_arr, t_ref)`` on the host
(numpy, float64) and ``encode(t_ref)``, the constants of the device kernel
that evaluates the same expressions per sample (``csrc/pulse.cu``). The
device evaluation is bit-identical for ``DerivativeModulating`` and agrees to
the last few ulps of ``sin``/``cos``/``atan``/``pow`` for the others. Any
other object with a ``generate`` method is evaluated on the host and passed
as a proper-time table.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from pyloki_gb300 import _lib
from pyloki_gb300.config import C_VAL


def _fact(k: np.ndarray) -> np.ndarray:
    return np.array([float(math.factorial(int(i))) for i in np.ravel(k)]).reshape(np.shape(k))


def _encode(kind: str, t_ref: float, coeffs) -> _lib.LokiModulation:
    m = _lib.LokiModulation()
    m.kind = _lib.MOD_KINDS[kind]
    c = np.asarray(coeffs, dtype=np.float64)
    if len(c) > _lib.MOD_MAX_COEFFS:
        msg = f"at most {_lib.MOD_MAX_COEFFS} modulation coefficients"
        raise ValueError(msg)
    m.ncoeff = len(c)
    m.t_ref = float(t_ref)
    for i, v in enumerate(c):
        m.c[i] = float(v)
    return m


@dataclass
class DerivativeModulating:
    """Taylor line-of-sight displacement about ``t_ref`` up to snap, in m/s^k
    (``simulation/modulate.py:23-50``)."""

    shift: float = 0.0
    vel: float = 0.0
    acc: float = 0.0
    jerk: float = 0.0
    snap: float = 0.0

    def generate(self, t_arr: np.ndarray, t_ref: float = 0.0) -> np.ndarray:
        dt = np.asarray(t_arr, dtype=np.float64) - t_ref
        inner = self.jerk * (1.0 / 6.0) + dt * self.snap * (1.0 / 24.0)
        delay = self.shift + dt * (self.vel + dt * (self.acc * 0.5 + dt * inner))
        return t_arr - delay / C_VAL

    def encode(self, t_ref: float) -> _lib.LokiModulation:
        return _encode("derivative", t_ref, [self.shift, self.vel, self.acc, self.jerk,
                                             self.snap])

    def to_circular(self) -> dict[str, float]:
        """Circular-orbit parameters with the same acc, jerk and snap
        (``modulate.py:52-70``)."""
        if self.acc == 0.0 and self.snap == 0.0:
            msg = "Degenerate phase: cannot recover omega from (d2,d3,d4)."
            raise ValueError(msg)
        if self.acc * self.snap >= 0.0:
            msg = "Incompatible with circular orbit: require d2*d4<0."
            raise ValueError(msg)
        omega = np.sqrt(-self.snap / self.acc)
        x_sin = -self.acc / (C_VAL * omega**2)
        x_cos = -self.jerk / (C_VAL * omega**3)
        return {"p_orb": 2.0 * np.pi / omega, "psi": float(np.arctan2(x_sin, x_cos)),
                "x_orb": float(np.hypot(x_sin, x_cos))}


@dataclass
class DerivativeSeriesModulating:
    """Taylor displacement with any number of derivatives ``coeffs[k]`` (m/s^k)
    (``simulation/modulate.py:73-108``)."""

    coeffs: np.ndarray = field(default_factory=lambda: np.zeros(1))

    @property
    def order(self) -> int:
        return len(self.coeffs) - 1

    def _norm(self) -> np.ndarray:
        k = np.arange(self.order + 1)
        return np.asarray(self.coeffs, dtype=np.float64) / _fact(k)

    def generate(self, t_arr: np.ndarray, t_ref: float = 0.0) -> np.ndarray:
        k = np.arange(self.order + 1)
        powers = (np.asarray(t_arr, dtype=np.float64) - t_ref)[None, :] ** k[:, None]
        delay = np.sum(self._norm()[:, None] * powers, axis=0)
        return t_arr - delay / C_VAL

    def encode(self, t_ref: float) -> _lib.LokiModulation:
        return _encode("derivative_series", t_ref, self._norm())


@dataclass
class CircularModulating:
    """Circular Keplerian orbit: ``x_orb`` light-seconds, or masses
    (``simulation/modulate.py:111-165``)."""

    p_orb: float
    psi: float
    x_orb: float | None = None
    m_c: float | None = None
    m_p: float = 1.4
    sin_i: float = 1.0

    def __post_init__(self) -> None:
        if self.x_orb is None and self.m_c is not None:
            a = 0.005 * ((self.m_p + self.m_c) * self.p_orb**2) ** (1 / 3)
            self.x_orb = a * (self.m_c / (self.m_p + self.m_c)) * self.sin_i
        if self.x_orb is None:
            msg = "CircularModulating needs x_orb or m_c"
            raise ValueError(msg)

    def generate(self, t_arr: np.ndarray, t_ref: float = 0.0) -> np.ndarray:
        omega = 2 * np.pi / self.p_orb
        return t_arr - self.x_orb * np.sin(omega * (t_arr - t_ref) + self.psi)

    def encode(self, t_ref: float) -> _lib.LokiModulation:
        return _encode("circular", t_ref, [self.x_orb, 2 * np.pi / self.p_orb, self.psi])

    def to_derivatives(self) -> dict[str, float]:
        """Displacement derivatives at ``t_ref`` (``modulate.py:142-165``)."""
        omega = 2.0 * np.pi / self.p_orb
        xs, xc = self.x_orb * np.sin(self.psi), self.x_orb * np.cos(self.psi)
        d2 = -C_VAL * xs * omega**2
        d3 = -C_VAL * xc * omega**3
        return {"shift": C_VAL * xs, "vel": C_VAL * xc * omega, "acc": d2, "jerk": d3,
                "snap": -d2 * omega**2, "crackle": -d3 * omega**2}


@dataclass
class CircularT0Modulating:
    """Circular orbit with a reference epoch ``t0`` (``modulate.py:201-213``)."""

    a: float
    p_orb: float
    t0: float

    def _phi(self, t_ref: float) -> float:
        return 2 * np.pi * ((t_ref - self.t0) % self.p_orb) / self.p_orb

    def generate(self, t_arr: np.ndarray, t_ref: float = 0.0) -> np.ndarray:
        omega = 2 * np.pi / self.p_orb
        delay = self.a * np.sin(omega * (t_arr - t_ref) + self._phi(t_ref))
        return t_arr - delay / C_VAL

    def encode(self, t_ref: float) -> _lib.LokiModulation:
        return _encode("circular_t0", t_ref, [self.a, 2 * np.pi / self.p_orb, self._phi(t_ref)])


def keplerian_nu(t_arr: np.ndarray, p_orb: float, ecc: float, phi: float,
                 n_iters: int = 8) -> np.ndarray:
    """True anomaly from 8 Newton steps on Kepler's equation started at the
    mean anomaly (``kepler.py:63-101``)."""
    m_arr = 2 * np.pi * ((t_arr % p_orb) / p_orb) + phi
    e_arr = m_arr.copy()
    for _ in range(n_iters):
        e_arr += (m_arr + ecc * np.sin(e_arr) - e_arr) / (1 - ecc * np.cos(e_arr))
    return 2 * np.arctan(np.sqrt((1 + ecc) / (1 - ecc)) * np.tan(e_arr / 2))


@dataclass
class KeplerianModulating:
    """Eccentric orbit: projected z of ``kepler.keplerian_z``
    (``modulate.py:216-236``, ``kepler.py:104-140``)."""

    p_orb: float
    ecc: float
    phi: float
    a: float
    om: float
    inc: float

    def generate(self, t_arr: np.ndarray, t_ref: float = 0.0) -> np.ndarray:
        ecc = abs(self.ecc)
        nu = keplerian_nu(t_arr - t_ref, self.p_orb, ecc, self.phi)
        r = self.a * (1 - ecc**2) / (1 + ecc * np.cos(nu))
        return t_arr - r * np.sin(nu + self.om) * np.sin(self.inc) / C_VAL

    def encode(self, t_ref: float) -> _lib.LokiModulation:
        ecc = abs(self.ecc)
        return _encode("keplerian", t_ref, [self.p_orb, ecc, self.phi, self.a * (1 - ecc**2),
                                            self.om, np.sin(self.inc),
                                            np.sqrt((1 + ecc) / (1 - ecc)), 1.0 / self.p_orb])


type_to_mods: dict[str, type] = {
    "derivative": DerivativeModulating,
    "derivative_series": DerivativeSeriesModulating,
    "circular": CircularModulating,
    "circular_t0": CircularT0Modulating,
    "keplerian": KeplerianModulating,
}

"""Oracle (test infrastructure only) for the synthetic pulsar generator.

A numpy restatement of pyloki's ``PulseSignalConfig.generate``
(``simulation/pulse.py:310-406``) and the pieces it calls. Only the tests and
the CPU-baseline leg of the benchmark use it, as the checker; nothing on the
product path imports it.

- proper time: ``simulation/modulate.py`` (derivative 36-50, series 77-82,
  circular 136-140, circular_t0 208-213, keplerian 226-236 with
  ``kepler.py:63-140``);
- CDF table: ``build_cdf_lut`` (pulse.py:13-35);
- template: ``generate_pulse_template`` (pulse.py:38-68), float64 with the
  reference's operation order;
- fold bins: ``get_phase_idx_int`` (utils/psr_utils.py:12-56);
- folds: ``brutefold`` (core/fold.py:57-105) with one segment; float32
  sequential sums as the reference, or exact float64 sums;
- calibration: pulse.py:380-400 and ``calibrate_scale_on_folds``
  (pulse.py:71-118) with ``boxcar_snr_1d`` (detection/scoring.py:43-140),
  float32 where the reference is float32.
"""

from __future__ import annotations

import math

import numpy as np
from scipy import stats

C_VAL = 299792458.0


def cdf_lut(shape: str, width: float, pos: float, ngrid: int = 4096) -> np.ndarray:
    phase = np.linspace(0.0, 1.0, ngrid, endpoint=False)
    if shape == "boxcar":
        rv = stats.uniform(loc=pos, scale=width)
    elif shape == "gaussian":
        rv = stats.norm(loc=pos, scale=width / (2 * np.sqrt(2 * np.log(10))))
    elif shape == "von_mises":
        rv = stats.vonmises(loc=pos, kappa=np.log(2.0) / (2.0 * np.sin(np.pi * width / 2.0) ** 2))
    else:
        raise ValueError(shape)
    cdf = rv.cdf(phase).astype(np.float64)
    return np.concatenate([cdf, cdf[:1]]).astype(np.float32)


def proper_time(kind: str, params: dict, nsamps: int, dt: float, t_ref: float) -> np.ndarray:
    t = np.arange(nsamps, dtype=np.float64) * dt
    d = t - t_ref
    if kind == "derivative":
        p = {k: params.get(k, 0.0) for k in ("shift", "vel", "acc", "jerk", "snap")}
        delay = p["shift"] + d * (p["vel"] + d * (p["acc"] * 0.5 + d * (
            p["jerk"] * (1.0 / 6.0) + d * p["snap"] * (1.0 / 24.0))))
        return t - delay / C_VAL
    if kind == "derivative_series":
        c = np.asarray(params["coeffs"], np.float64)
        k = np.arange(len(c))
        norm = c / np.array([float(math.factorial(int(i))) for i in k])
        return t - np.sum(norm[:, None] * d[None, :] ** k[:, None], axis=0) / C_VAL
    if kind == "circular":
        omega = 2 * np.pi / params["p_orb"]
        return t - params["x_orb"] * np.sin(omega * d + params["psi"])
    if kind == "circular_t0":
        omega = 2 * np.pi / params["p_orb"]
        phi = 2 * np.pi * ((t_ref - params["t0"]) % params["p_orb"]) / params["p_orb"]
        return t - params["a"] * np.sin(omega * d + phi) / C_VAL
    if kind == "keplerian":
        ecc = abs(params["ecc"])
        p_orb = params["p_orb"]
        m = 2 * np.pi * ((d % p_orb) / p_orb) + params["phi"]
        e = m.copy()
        for _ in range(8):
            e += (m + ecc * np.sin(e) - e) / (1 - ecc * np.cos(e))
        nu = 2 * np.arctan(np.sqrt((1 + ecc) / (1 - ecc)) * np.tan(e / 2))
        r = params["a"] * (1 - ecc**2) / (1 + ecc * np.cos(nu))
        return t - r * np.sin(nu + params["om"]) * np.sin(params["inc"]) / C_VAL
    raise ValueError(kind)


def template(pt: np.ndarray, dt: float, period: float, lut: np.ndarray) -> np.ndarray:
    ngrid = lut.shape[0] - 1
    lut64 = lut.astype(np.float64)
    inv = 1.0 / period
    p0 = np.mod(pt, period) * inv
    p1 = np.mod(pt + dt, period) * inv

    def at(p):
        x = p * ngrid
        i = np.clip(x.astype(np.int64), 0, ngrid - 1)
        f = x - i
        return (1.0 - f) * lut64[i] + f * lut64[i + 1]

    return np.where(p1 > p0, at(p1) - at(p0), 0.0).astype(np.float32)


def phase_bins(pt: np.ndarray, freq: float, nbins: int) -> np.ndarray:
    phase = pt * freq
    phase = phase - np.floor(phase)
    iphase = phase * nbins
    iphase = np.where(iphase >= nbins, 0.0, iphase)
    ib = (iphase.astype(np.float32) + np.float32(0.5)).astype(np.int64)
    return np.where(ib == nbins, 0, ib)


def fold_f32(values: np.ndarray, bins: np.ndarray, nbins: int) -> np.ndarray:
    """Sequential float32 sums in sample order (the reference's brutefold)."""
    out = np.zeros(nbins, np.float32)
    order = np.argsort(bins, kind="stable")
    b = bins[order]
    v = values[order].astype(np.float32)
    starts = np.searchsorted(b, np.arange(nbins))
    ends = np.searchsorted(b, np.arange(nbins), side="right")
    for k in range(nbins):
        if ends[k] > starts[k]:
            out[k] = np.cumsum(v[starts[k]:ends[k]], dtype=np.float32)[-1]
    return out


def fold_exact(values: np.ndarray, bins: np.ndarray, nbins: int) -> np.ndarray:
    """Float64 sums (exact for float32 inputs of the generator's ranges up to
    the float64 rounding of the total)."""
    return np.bincount(bins, weights=values.astype(np.float64), minlength=nbins)


def boxcar_max_f32(x: np.ndarray) -> np.float32:
    """max over widths 1 .. n/2 - 1 of boxcar_snr_1d (stdnoise 1)."""
    x = np.asarray(x, np.float32)
    n = len(x)
    wmax = n // 2 - 1
    p = np.empty(n + wmax, np.float32)
    p[:n] = np.cumsum(x, dtype=np.float32)
    p[n:] = p[:wmax] + p[n - 1]
    total = np.float64(p[n - 1])
    best = -np.inf
    for w in range(1, wmax + 1):
        dmax = np.max(p[w:w + n] - p[:n])
        size_w = np.float64(np.float32(n - w))
        h = np.sqrt(size_w / (n * w))
        b = w * h / size_w
        best = max(best, np.float32((h + b) * np.float64(dmax) - b * total))
    return np.float32(best)


def off_pulse_mask(nbins: int, ducy: float, phi0: float) -> np.ndarray:
    center = round(phi0 * nbins) % nbins
    width = max(1, round(ducy * nbins))
    on = (center - width // 2 + np.arange(width)) % nbins
    mask = np.ones(nbins, dtype=bool)
    mask[on] = False
    return mask


def calibrate(noise_vals, noise_var, tmpl_vals, snr: float, ducy: float, phi0: float,
              max_iter: int = 5, tol: float = 1e-2):
    """(noise_scale, signal scale, template S/N, last measured S/N) from
    float32 folds."""
    vals = np.asarray(noise_vals, np.float32)
    var = np.asarray(noise_var, np.float32)
    tm = np.asarray(tmpl_vals, np.float32)
    nbins = len(vals)
    off = off_pulse_mask(nbins, ducy, phi0)
    sd = np.std(vals[off])  # float32, as the reference
    ns = np.float32(np.float32(1.0) / sd)
    vals_s = (vals * ns).astype(np.float32)
    var_s = (var * np.float32(ns * ns)).astype(np.float32)
    root = np.sqrt(var_s)
    tn = (tm / root).astype(np.float32)
    nn = (vals_s / root).astype(np.float32)
    snr_t = boxcar_max_f32(tn)
    cur = float(np.float32(np.float32(snr) / snr_t) * ns)
    meas = np.nan
    for _ in range(max_iter):
        comb = (nn.astype(np.float64) + cur * tn.astype(np.float64)).astype(np.float32)
        meas = float(boxcar_max_f32(comb))
        diff = meas - snr
        if diff * diff < tol * tol:
            break
        cur -= 0.8 * diff / float(snr_t)
    return float(ns), cur, float(snr_t), meas


def emit(noise: np.ndarray, tmpl: np.ndarray, ns: float, scale: float):
    ns32 = np.float32(ns)
    ts_e = (ns32 * noise.astype(np.float32) + np.float32(scale) * tmpl).astype(np.float32)
    ts_v = np.full(len(noise), ns32 * ns32, np.float32)
    return ts_e, ts_v


def generate(period: float, dt: float, nsamps: int, snr: float, ducy: float, noise: np.ndarray,
             *, shape: str = "gaussian", phi0: float = 0.5, kind: str = "derivative",
             params: dict | None = None, t_ref: float | None = None, max_iter: int = 5,
             tol: float = 1e-2, exact_folds: bool = False) -> dict:
    t_ref = nsamps * dt / 2 if t_ref is None else t_ref
    lut = cdf_lut(shape, ducy, phi0, max(4096, int(100 / ducy)))
    pt = proper_time(kind, params or {}, nsamps, dt, t_ref)
    tm = template(pt, dt, period, lut)
    nbins = int(period / dt)
    bins = phase_bins(pt, 1.0 / period, nbins)
    fold = fold_exact if exact_folds else fold_f32
    folds = np.stack([fold(noise, bins, nbins), np.bincount(bins, minlength=nbins),
                      fold(tm, bins, nbins)]).astype(np.float32)
    ns, scale, snr_t, meas = calibrate(folds[0], folds[1], folds[2], snr, ducy, phi0,
                                       max_iter, tol)
    ts_e, ts_v = emit(noise, tm, ns, scale)
    return {"proper_time": pt, "template": tm, "bins": bins, "folds": folds, "noise_scale": ns,
            "scale": scale, "snr_template": snr_t, "snr_measured": meas, "ts_e": ts_e,
            "ts_v": ts_v, "lut": lut}


def load_case(path) -> dict:
    """A generator fixture as keyword arguments of ``generate`` plus the
    reference's outputs."""
    z = np.load(path)
    params, off = {}, 0
    for name, size in zip(z["param_names"].tolist(), z["param_sizes"].tolist()):
        v = z["param_values"][off:off + size]
        params[name] = v if name == "coeffs" else float(v[0])
        off += size
    case = {k: z[k] for k in z.files}
    case["params"] = params
    return case

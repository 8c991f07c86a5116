"""Oracle (test infrastructure only) for the alternative profile scorers of
``detection/scoring.py``: plain-Python / numpy restatements used by the tests
as the checker. Nothing on the product path imports it.

- ``kadane``: ``kadane_circular_normalized_1d`` (scoring.py:675-755),
  float64 scalar loop;
- ``snr_e_mat_2d``: ``compute_snr_e_mat_2d`` (scoring.py:491-524);
- ``snr_double``: ``_compute_snr_double`` (scoring.py:561-627) with the
  table lookups of ``utils/maths.py:80-101``;
- ``harmonic``: ``harmonic_summing_score_func`` (scoring.py:630-642).
"""

from __future__ import annotations

import numpy as np
from scipy import stats

CHI_RES, CHI_MAX, ISF_RES, ISF_MAX = 0.5, 300.0, 0.1, 400.0


def tables() -> tuple[np.ndarray, np.ndarray]:
    x = np.arange(0, CHI_MAX, CHI_RES)
    chi = np.zeros((65, len(x)))
    for i in range(1, 65):
        chi[i] = -stats.chi2.logsf(x, i)
    isf = stats.norm.isf(np.exp(-np.arange(0, ISF_MAX, ISF_RES)))
    return chi, isf


def chi_minus_logsf(chi: np.ndarray, x: float, df: int) -> float:
    flat = np.append(chi.ravel(), 0.0)
    if x < CHI_MAX:
        pos = x / CHI_RES
        fr = pos % 1
        i = df * chi.shape[1] + int(pos)
        return flat[i] * (1 - fr) + flat[i + 1] * fr
    return chi[df, -1] * x / CHI_MAX


def norm_isf(isf: np.ndarray, m: float) -> float:
    """Negative positions index from the end of the table, as the reference's
    do (a weak candidate's score wraps to the top of the table)."""
    if m < ISF_MAX:
        pos = m / ISF_RES
        fr = pos % 1
        i = int(pos)
        j = min(i + 1, len(isf) - 1)
        return isf[i] * (1 - fr) + isf[j] * fr
    return isf[-1] * (m / ISF_MAX) ** 0.5


def kadane(x: np.ndarray, biases: np.ndarray) -> tuple[float, int, int]:
    size = len(x)
    mean = sum(float(v) for v in x) / size
    best, best_w, best_s = -np.finfo(np.float64).max, 1, 0
    for bias in (float(b) for b in biases):
        max_sum, cur_max, s_max, e_max, t_max = -np.finfo(np.float64).max, 0.0, 0, 0, 0
        min_sum, cur_min, s_min, e_min, t_min = np.finfo(np.float64).max, 0.0, 0, 0, 0
        for i in range(size):
            val = float(x[i]) - mean - bias
            cur_max += val
            if cur_max > max_sum:
                max_sum, s_max, e_max = cur_max, t_max, i
            if cur_max < 0.0:
                cur_max, t_max = 0.0, i + 1
            cur_min += val
            if cur_min < min_sum:
                min_sum, s_min, e_min = cur_min, t_min, i
            if cur_min > 0.0:
                cur_min, t_min = 0.0, i + 1
        biased, start, width = max_sum, s_max, e_max - s_max + 1
        wrapped_w = size - (e_min - s_min + 1)
        if wrapped_w > 0:
            wrapped = (-size * bias) - min_sum
            if wrapped > biased:
                biased, start, width = wrapped, (e_min + 1) % size, wrapped_w
        unbiased = biased + width * bias
        snr = unbiased * np.sqrt(size / (width * (size - width))) if 0 < width < size else 0.0
        if snr > best:
            best, best_w, best_s = float(snr), width, start
    return best, best_w, best_s


def snr_e_mat_2d(prof: np.ndarray, e_mat: np.ndarray, shifts: np.ndarray,
                 stdnoise: float = 1.0) -> np.ndarray:
    proj = np.dot(prof.astype(np.float32), e_mat.T)
    nsh = e_mat.shape[1] // shifts
    edges = np.concatenate([[0], np.cumsum(nsh)])
    return np.stack([proj[:, a:b].max(axis=1) / stdnoise
                     for a, b in zip(edges[:-1], edges[1:])], axis=1).astype(np.float32)


def snr_double(prof: np.ndarray, e_mat: np.ndarray, n_corr: int = 10) -> np.ndarray:
    scores = np.stack([np.dot(e_mat, x.astype(np.float32)) for x in prof])
    return snr_double_from_scores(scores, np.dot(e_mat, e_mat.T), n_corr)


def snr_double_from_scores(scores: np.ndarray, inner: np.ndarray,
                           n_corr: int = 10) -> np.ndarray:
    """The two-peak score from given projections (n, nfilt)."""
    chi, isf = tables()
    nf = scores.shape[1]
    lee_d, lee_s = np.log2((nf * nf - 1) / 2), np.log2(nf)
    out = np.empty(len(scores), np.float32)
    for p, row in enumerate(scores):
        sc = np.asarray(row, np.float32).astype(np.float64)
        single = float(sc.max()) ** 2
        good = np.argsort(sc, kind="stable")[-n_corr:]
        dbl, s = single, 0.0
        for i in range(n_corr - 1):
            for j in range(i + 1, n_corr):
                a, b = good[i], good[j]
                g = float(inner[a, b])
                if abs(g) < 0.99:
                    s = (sc[a] ** 2 + sc[b] ** 2 - 2 * g * sc[a] * sc[b]) / (1 - g**2)
                dbl = max(s, dbl)
        x1 = chi_minus_logsf(chi, single, 1) - lee_s
        x2 = chi_minus_logsf(chi, dbl, 2) - lee_d
        out[p] = norm_isf(isf, max(x1, x2))
    return out


def harmonic(fold: np.ndarray, n_harmonics: int) -> float:
    chi, isf = tables()
    e, v = fold
    f = (e / np.sqrt(v)).astype(np.float64)
    ft = np.fft.fft(f) / np.sqrt(len(f))
    best, raw = -np.inf, 0.0
    for i in range(1, n_harmonics + 1):
        raw += abs(ft[i]) ** 2
        best = max(chi_minus_logsf(chi, raw * 2, 2 * i), best)
    return norm_isf(isf, best)


def snr_fft(prof: np.ndarray, templates: np.ndarray) -> np.ndarray:
    """``_compute_snr_fft``: circular pad to a power of two, zero-padded
    templates, irfft(rfft(x) rfft(t)), max over the first nbins lags."""
    nb = prof.shape[-1]
    n = 1 << int(np.ceil(np.log2(nb)))
    xx = np.concatenate([prof, prof[:, :n - nb]], axis=1).astype(np.float32)
    yy = np.concatenate([templates, np.zeros((len(templates), n - nb))], axis=1)
    fx, fy = np.fft.rfft(xx), np.fft.rfft(yy)
    return np.array([[np.fft.irfft(fx[p] * fy[t], n)[:nb].max() for t in range(len(templates))]
                     for p in range(len(prof))], np.float32)

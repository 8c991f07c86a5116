"""Chebyshev-basis host math for the enumerate-prune tree.

The small (P+1) x (P+1) matrices that the GPU kernels apply per leaf are
built here, once per level, with the reference's formulas and the same
floating-point operation order (``utils/maths.py:401-589``), so the kernels
see bit-identical constants. Leaf transforms that touch every survivor once
per run (seed and report) are done with numpy exactly as the reference does
(``core/chebyshev.py:14-70,380-404``, ``utils/transforms.py:458-620``).

Coefficient order follows the reference: leaves hold [alpha_P, ..., alpha_0].
"""

from __future__ import annotations

import numpy as np

from pyloki_gb300.config import C_VAL, fact


def nbinom(n: int, k: int) -> int:
    """Integer binomial coefficient (``utils/maths.py:37-53``)."""
    if k < 0 or k > n:
        return 0
    if k in (0, n):
        return 1
    k = min(k, n - k)
    if n <= 120:
        return int(fact(n)) // (int(fact(k)) * int(fact(n - k)))
    out = 1
    for i in range(k):
        out = out * (n - i) // (i + 1)
    return out


def conn_s(k: int, m: int) -> float:
    """Power series -> Chebyshev connection coefficient S_{k,m} (maths.py:401-423)."""
    if k < 0 or m < 0 or m > k or (k - m) % 2 != 0:
        return 0.0
    n = (k - m) // 2
    delta = 1 if m == 0 else 0
    return 2.0 ** (1 - k - delta) * nbinom(k, n)


def conn_r(k: int, m: int) -> float:
    """Chebyshev -> power series connection coefficient R_{k,m} (maths.py:426-448)."""
    if k < 0 or m < 0 or m > k or (k - m) % 2 != 0:
        return 0.0
    if m == 0 and k % 2 == 0:
        return (-1) ** (k // 2)
    n = (k - m) // 2
    r = (k + m) // 2
    return ((-1) ** n) * (2.0 ** (m - 1)) * (2.0 * k / (k + m)) * nbinom(r, n)


def transform_coeff(n: int, k: int, p: float, q: float) -> float:
    """C_{n,k}(p, q) of a domain change (maths.py:451-482)."""
    if k > n:
        return 0.0
    result = 0.0
    for m in range(k, n + 1):
        r_nm = conn_r(n, m)
        inner = 0.0
        for i in range(k, m + 1):
            inner += nbinom(m, i) * p**i * q ** (m - i) * conn_s(i, k)
        result += r_nm * inner
    return result


def conn_matrix_s(k_max: int) -> np.ndarray:
    out = np.zeros((k_max + 1, k_max + 1), np.float64)
    for k in range(k_max + 1):
        for m in range(k + 1):
            out[k, m] = conn_s(k, m)
    return out


def conn_matrix_r(k_max: int) -> np.ndarray:
    out = np.zeros((k_max + 1, k_max + 1), np.float64)
    for k in range(k_max + 1):
        for m in range(k + 1):
            out[k, m] = conn_r(k, m)
    return out


def transform_matrix(poly_order: int, tc1: float, ts1: float, tc2: float,
                     ts2: float) -> np.ndarray:
    """Descending-order C for coefficients on (tc1, ts1) -> (tc2, ts2), so that
    ``alpha_new = alpha @ C`` (maths.py:534-589, coeff_order=1)."""
    if ts1 <= 0 or ts2 <= 0:
        msg = "ts1 and ts2 must be positive."
        raise ValueError(msg)
    p = ts2 / ts1
    q = (tc2 - tc1) / ts1
    size = poly_order + 1
    out = np.zeros((size, size), np.float64)
    for i in range(size):
        n = poly_order - i
        for j in range(size):
            out[i, j] = transform_coeff(n, poly_order - j, p, q)
    return out


def taylor_to_cheby_full(taylor_full: np.ndarray, t_s: float) -> np.ndarray:
    """(..., n, 2) Taylor values/errors -> Chebyshev (transforms.py:458-488)."""
    if t_s <= 0:
        msg = "t_s must be a positive."
        raise ValueError(msg)
    n = taylor_full.shape[-2]
    s_mat = conn_matrix_s(n - 1)
    k = np.arange(n, dtype=np.int64)
    scale = t_s**k / fact(k)
    vals = np.ascontiguousarray(taylor_full[..., ::-1, 0]) * scale
    errs = np.ascontiguousarray(taylor_full[..., ::-1, 1]) * scale
    out = np.empty_like(taylor_full)
    out[..., :, 0] = (vals @ s_mat)[..., ::-1]
    out[..., :, 1] = np.sqrt(errs**2 @ s_mat**2)[..., ::-1]
    return out


def cheby_to_taylor_full(alpha_full: np.ndarray, t_s: float) -> np.ndarray:
    """(..., n, 2) Chebyshev values/errors -> Taylor (transforms.py:587-620)."""
    if t_s <= 0:
        msg = "t_s must be a positive."
        raise ValueError(msg)
    n = alpha_full.shape[-2]
    vals = np.ascontiguousarray(alpha_full[..., ::-1, 0])
    errs = np.ascontiguousarray(alpha_full[..., ::-1, 1])
    r_mat = conn_matrix_r(n - 1)
    d_vals = vals @ r_mat
    var_d = errs**2 @ r_mat**2
    k = np.arange(n, dtype=np.int64)
    scale = fact(k) / t_s**k
    out = np.empty_like(alpha_full)
    out[..., :, 0] = (d_vals * scale)[..., ::-1]
    out[..., :, 1] = np.sqrt(var_d * scale**2)[..., ::-1]
    return out


def seed_leaves(param_arr, dparams: np.ndarray, poly_order: int,
                scale_init: float) -> np.ndarray:
    """Seed leaves in the Chebyshev basis (core/chebyshev.py:14-70)."""
    mesh = np.meshgrid(*param_arr, indexing="ij")
    cart = np.stack([m.ravel() for m in mesh], axis=1)
    n = cart.shape[0]
    dparams = np.asarray(dparams, np.float64)
    f0 = cart[:, -1]
    leaves_d = np.zeros((n, poly_order + 1, 2), np.float64)
    leaves_d[:, :-2, 0] = cart[:, :-1]
    leaves_d[:, :-2, 1] = dparams[:-1]
    leaves_d[:, -2, 1] = dparams[-1] * (C_VAL / f0)
    leaves = np.zeros((n, poly_order + 2, 2), np.float64)
    leaves[:, :-1] = taylor_to_cheby_full(leaves_d, scale_init)
    leaves[:, -1, 0] = f0
    return leaves


def report_batch(leaves: np.ndarray, coord_report: tuple[float, float]) -> np.ndarray:
    """Final parameters in the Taylor basis at the report domain
    (core/chebyshev.py:380-404)."""
    _, scale = coord_report
    out = leaves.copy()
    f0 = leaves[:, -1, 0]
    d = cheby_to_taylor_full(leaves[:, :-1, :], scale)
    vals = d[:, :-2, 0]
    sigs = d[:, :-2, 1]
    out[:, -2, 0] = d[:, -1, 0]
    out[:, -2, 1] = d[:, -1, 1]
    v_final = d[:, -2, 0]
    dv_final = d[:, -2, 1]
    s = 1 - v_final / C_VAL
    out[:, :-3, 0] = vals / s[:, None]
    out[:, :-3, 1] = np.sqrt((sigs / s[:, None]) ** 2
                             + ((vals / (C_VAL * s[:, None] ** 2)) ** 2) * (dv_final[:, None] ** 2))
    out[:, -3, 0] = f0 * s
    out[:, -3, 1] = f0 * dv_final / C_VAL
    return out

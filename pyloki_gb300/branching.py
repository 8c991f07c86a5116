"""Branching pattern of an enumerate-prune run (``config.py:758-819``).

The average number of children per parent at every pruning level of a Taylor
tree, tracked per final FFA frequency from the FFA's grid steps, with no
threshold applied: the input of the threshold-scheme design
(``detection/thresholding.py``). Host-side FP64 with the reference's
operation order (``core/taylor.py:415-492``), vectorised over frequencies.
"""

from __future__ import annotations

import numpy as np

from pyloki_gb300.config import C_VAL, FLOAT_EPSILON, fact, poly_taylor_step_f
from pyloki_gb300.scheme import MiddleOutScheme


def _taylor_factors(n_params: int, tobs: float, nbins: int, use_cheby: bool) -> np.ndarray:
    """Per-parameter bin-shift factors of ``poly_taylor_shift_d_vec``
    (``utils/psr_utils.py:227-248``) before the frequency scale."""
    k = np.arange(n_params - 1, -1, -1)
    factors = (tobs - 0) ** (k + 1) * nbins / fact(k + 1)
    if use_cheby:
        factors = factors / 2**k
    return factors


def shift_taylor_errors(errors: np.ndarray, delta_t: float,
                        tiling_strategy: str = "aggressive") -> np.ndarray:
    """Taylor errors re-referenced by ``delta_t`` (``utils/transforms.py:51-90``)."""
    n = errors.shape[-1]
    powers = np.tril(np.arange(n)[:, np.newaxis] - np.arange(n))
    t_mat = delta_t**powers / fact(powers) * np.tril(np.ones_like(powers))
    errors = np.ascontiguousarray(errors)
    if tiling_strategy == "conservative":
        return errors @ np.abs(t_mat).T
    if tiling_strategy == "quadrature":
        return np.sqrt((errors**2) @ (t_mat**2).T)
    if tiling_strategy == "aggressive":
        return errors * np.abs(np.diag(t_mat))
    msg = f"Invalid tiling strategy: {tiling_strategy}"
    raise ValueError(msg)


def generate_bp_poly_taylor(param_arr, dparams_act: np.ndarray, tseg_ffa: float,
                            nsegments: int, nbins: int, eta: float, ref_seg: int, *,
                            use_moving_grid: bool = True,
                            tiling_strategy: str = "aggressive",
                            use_cheby_coarsening: bool = True) -> np.ndarray:
    """Children per parent at levels 1 .. nsegments - 1 of a Taylor tree
    seeded on the final FFA grid (``core/taylor.py:415-492``).

    Every final frequency starts with the FFA's actual steps (the frequency
    step expressed as a velocity step, dv = df * c / f0). At each level a
    parameter whose step shifts the profile by at least ``eta`` bins over the
    current span is split into ``ceil(step / new_step)`` children; the level's
    branching is the child count summed over the tree so far (weights =
    leaves per frequency) divided by the parent count.
    """
    n_params = len(dparams_act)
    f0 = np.asarray(param_arr[-1], dtype=np.float64)
    scheme = MiddleOutScheme(nsegments, ref_seg, tseg_ffa, stride=1)
    weights = np.ones(len(f0), dtype=np.float64)
    pattern = np.empty(nsegments - 1, dtype=np.float64)
    dcur = np.tile(np.asarray(dparams_act, dtype=np.float64), (len(f0), 1))
    dcur[:, n_params - 1] *= C_VAL / f0
    f_scale = (f0 / C_VAL)[:, np.newaxis]
    for level in range(1, nsegments):
        coord_next = scheme.get_coord(level)
        coord_cur = scheme.get_current_coord(level, moving_grid=use_moving_grid)
        tobs = coord_cur[1]
        step_f = poly_taylor_step_f(n_params, tobs, nbins, eta, t_ref=0,
                                    use_cheby=use_cheby_coarsening)
        dnew = step_f[np.newaxis, :] * C_VAL / f0[:, np.newaxis]
        factors = np.broadcast_to(_taylor_factors(n_params, tobs, nbins, use_cheby_coarsening),
                                  dcur.shape) * f_scale
        shift_bins = np.abs(dcur - dnew) * factors
        split = shift_bins >= (eta - FLOAT_EPSILON)
        nsplit = np.where(split, np.maximum(1, np.ceil(dcur / dnew - FLOAT_EPSILON)), 1.0)
        n_branches = np.prod(nsplit.astype(np.int64), axis=1)
        dnext = np.where(split, dcur / nsplit, dcur)
        pattern[level - 1] = np.sum(weights * n_branches) / np.sum(weights)
        weights = weights * n_branches
        if use_moving_grid:
            d_vec = np.zeros((len(f0), n_params + 1), dtype=np.float64)
            d_vec[:, :-1] = dnext
            dcur = shift_taylor_errors(d_vec, coord_next[0] - coord_cur[0],
                                       tiling_strategy)[:, :-1]
        else:
            dcur = dnext
    return pattern


def generate_branching_pattern(cfg, kind: str = "poly_taylor_moving", ref_seg: int = 0,
                               use_cheby_coarsening: bool = True) -> np.ndarray:
    """``PulsarSearchConfig.generate_branching_pattern`` (``config.py:758-819``)
    for the Taylor kinds ``"poly_taylor_moving"`` and ``"poly_taylor_fixed"``."""
    kinds = {"poly_taylor_moving": True, "poly_taylor_fixed": False}
    if kind not in kinds:
        msg = f"Invalid kind: {kind}"
        raise ValueError(msg)
    nsegments = int(np.ceil(cfg.nsamps / cfg.bseg_ffa))
    n = cfg.niters_ffa
    dparams = cfg.get_dparams(n, use_cheby_coarsening)
    return generate_bp_poly_taylor(
        cfg.get_param_arr(dparams), cfg.get_dparams_actual(n, use_cheby_coarsening),
        cfg.tseg_ffa, nsegments, cfg.nbins, cfg.eta, ref_seg, use_moving_grid=kinds[kind],
        tiling_strategy=cfg.tiling_strategy, use_cheby_coarsening=use_cheby_coarsening)


__all__ = ["generate_bp_poly_taylor", "generate_branching_pattern", "shift_taylor_errors"]

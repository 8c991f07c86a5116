"""Generate the golden FFA / scoring fixtures by running the pyloki reference.

Run in a container where the pyloki source tree is available (it is not on the
GPU test machines, which only read the committed ``.npz`` files):

    python tests/golden/make_fixtures.py /path/to/pyloki/src

The reference runs through ``refshim`` (numba replaced by plain Python), so
the fixtures carry numpy/IEEE semantics. Inputs are seeded; every fixture
stores its inputs, its configuration and the reference outputs.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _cfg_dict(cfg) -> dict:
    return {
        "nsamps": np.int64(cfg.nsamps),
        "tsamp": np.float64(cfg.tsamp),
        "nbins": np.int64(cfg.nbins),
        "eta": np.float64(cfg.eta),
        "param_limits": np.asarray(cfg.param_limits, dtype=np.float64),
        "ducy_max": np.float64(cfg.ducy_max),
        "wtsp": np.float64(cfg.wtsp),
        "bseg_brute": np.int64(cfg.bseg_brute),
        "bseg_ffa": np.int64(cfg.bseg_ffa),
    }


def _series(n: int, tsamp: float, freq: float, amp: float, seed: int):
    rng = np.random.default_rng(seed)
    t = np.arange(n) * tsamp
    phase = (t * freq) % 1.0
    pulse = np.exp(8.0 * (np.cos(2 * np.pi * (phase - 0.5)) - 1.0))
    ts_e = (rng.standard_normal(n) + amp * pulse).astype(np.float32)
    ts_v = (1.0 + 0.1 * rng.random(n)).astype(np.float32)
    return ts_e, ts_v


def ffa_case(name: str, n: int, limits, nbins: int, freq_inj: float, seed: int,
             ducy_max: float = 0.5, wtsp: float = 2.0) -> None:
    from pyloki.config import PulsarSearchConfig
    from pyloki.detection import scoring
    from pyloki.core.fold import ffa_taylor_resolve
    from pyloki.ffa import DynamicProgramming, FFAPlan
    from pyloki.utils.np_utils import cartesian_prod_st
    from pyloki.io.timeseries import TimeSeries

    tsamp = 64e-6
    ts_e, ts_v = _series(n, tsamp, freq_inj, 0.6, seed)
    cfg = PulsarSearchConfig(
        nsamps=n, tsamp=tsamp, nbins=nbins, eta=1.0,
        param_limits=np.asarray(limits, dtype=np.float64),
        ducy_max=ducy_max, wtsp=wtsp, use_fourier=False,
    )
    dyp = DynamicProgramming(TimeSeries(ts_e, ts_v, tsamp), cfg)
    dyp.initialize()
    out = {"ts_e": ts_e, "ts_v": ts_v, **_cfg_dict(cfg)}
    out["fold_0"] = dyp.fold.copy()
    for lvl in range(1, cfg.niters_ffa + 1):
        dyp._execute_iter()
        out[f"fold_{lvl}"] = dyp.fold.copy()
    out["niters"] = np.int64(cfg.niters_ffa)
    plan = FFAPlan(cfg)
    if cfg.nparams == 1:
        coords = plan.resolve_coordinates_freq()
        for lvl in range(1, cfg.niters_ffa + 1):
            out[f"plan_idx_{lvl}"] = coords[lvl]["idx"].copy()
            out[f"plan_shift_{lvl}"] = coords[lvl]["shift"].copy()
    # FFAPlan.resolve_coordinates fails for >1 parameter (it calls len() on the
    # integer grid counts), so the 4-field plan is taken from the resolve call
    # that unify_fold itself makes, flattened with C-order strides.
    for lvl in range(1, cfg.niters_ffa + 1):
        counts_prev = np.asarray(cfg.get_param_grid_count(lvl - 1), np.int64)
        strides = np.cumprod([1, *counts_prev[::-1][:-1]])[::-1]
        cart = cartesian_prod_st(cfg.get_param_arr(cfg.get_dparams(lvl)))
        rec = {k: [] for k in ("i_tail", "shift_tail", "i_head", "shift_head")}
        for pset in cart:
            it, st = ffa_taylor_resolve(pset, counts_prev, cfg.param_limits, lvl, 0,
                                        cfg.tseg_brute, cfg.nbins)
            ih, sh = ffa_taylor_resolve(pset, counts_prev, cfg.param_limits, lvl, 1,
                                        cfg.tseg_brute, cfg.nbins)
            rec["i_tail"].append(int(np.dot(it, strides)))
            rec["shift_tail"].append(st)
            rec["i_head"].append(int(np.dot(ih, strides)))
            rec["shift_head"].append(sh)
        out[f"plan_i_tail_{lvl}"] = np.asarray(rec["i_tail"], np.int64)
        out[f"plan_shift_tail_{lvl}"] = np.asarray(rec["shift_tail"], np.float64)
        out[f"plan_i_head_{lvl}"] = np.asarray(rec["i_head"], np.int64)
        out[f"plan_shift_head_{lvl}"] = np.asarray(rec["shift_head"], np.float64)
    for lvl in range(cfg.niters_ffa + 1):
        out[f"counts_{lvl}"] = np.asarray(cfg.get_param_grid_count(lvl), np.int64)
        for ip, arr in enumerate(cfg.get_param_arr(cfg.get_dparams(lvl))):
            out[f"param_{lvl}_{ip}"] = np.asarray(arr, np.float64)
        out[f"dparams_{lvl}"] = np.asarray(cfg.get_dparams(lvl), np.float64)
    widths = cfg.score_widths
    out["widths"] = widths
    folds_norm = dyp.get_fold_norm()
    out["fold_norm"] = folds_norm
    out["snrs"] = scoring.boxcar_snr_nd(folds_norm, widths, 1.0)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "levels", cfg.niters_ffa, "final", dyp.fold.shape,
          "bseg", cfg.bseg_brute)


def scoring_case(name: str, nbins: int, nprof: int, ducy_max: float, wtsp: float,
                 seed: int) -> None:
    from pyloki.detection import scoring

    rng = np.random.default_rng(seed)
    widths = scoring.generate_box_width_trials(nbins, ducy_max=ducy_max, wtsp=wtsp)
    prof = rng.standard_normal((nprof, nbins)).astype(np.float32)
    prof[: nprof // 4] += 3.0 * np.exp(
        -0.5 * ((np.arange(nbins) - nbins / 3) / 2.0) ** 2,
    ).astype(np.float32)
    snr = scoring.boxcar_snr_nd(prof, widths, 1.0)
    snr_std = scoring.boxcar_snr_nd(prof, widths, 1.7)
    comb = np.empty((nprof, 2, nbins), np.float32)
    comb[:, 0] = prof * 3.0
    comb[:, 1] = (9.0 + rng.random((nprof, nbins))).astype(np.float32)
    score = scoring.snr_score_batch_func(comb, widths)
    np.savez_compressed(
        HERE / f"{name}.npz", widths=widths, prof=prof, snr=snr, snr_std=snr_std,
        comb=comb, score=score,
    )
    print(name, widths)


def main() -> None:
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref_src = args[0] if args else "/root/reference/src"
    sys.path.insert(0, str(HERE))
    import refshim

    refshim.install(ref_src)
    import logging

    logging.disable(logging.CRITICAL)
    if "--skip-scoring" not in sys.argv:
        scoring_case("score_nb64", 64, 512, 0.5, 2.0, 11)
        scoring_case("score_nb50", 50, 256, 0.2, 1.5, 12)
        scoring_case("score_nb100", 100, 128, 0.3, 1.3, 13)
    ffa_case("ffa_freq", 2**15, [(10.0, 14.0)], 64, 12.3, 21)
    ffa_case("ffa_accel", 2**15, [(-3.0e5, 3.0e5), (200.0, 202.0)], 64, 201.1, 22)
    ffa_case("ffa_jerk", 2**15, [(-1.0e7, 1.0e7), (-3.0e5, 3.0e5), (200.0, 201.0)],
             50, 200.4, 23, ducy_max=0.2, wtsp=1.5)


if __name__ == "__main__":
    main()

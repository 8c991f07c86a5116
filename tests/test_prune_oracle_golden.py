"""The CPU pruning oracle against runs of the pyloki reference (no GPU).

Same fixtures and the same per-level checks as the GPU pruning tests: the
oracle is pinned to the reference before it is used to check anything else.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import load_golden

CASES = ["prune_taylor", "prune_taylor_fixed", "prune_taylor_cons", "prune_taylor_quad",
         "prune_taylor_overflow", "prune_cheby", "prune_cheby_fixed", "prune_cheby_cons",
         "prune_cheby_quad", "prune_circ", "prune_circ_b4", "prune_circ_quad",
         "prune_circ_fixed"]
TILING = {"prune_taylor_cons": "conservative", "prune_taylor_quad": "quadrature",
          "prune_cheby_cons": "conservative", "prune_cheby_quad": "quadrature",
          "prune_circ_quad": "quadrature"}


def _run(name):
    from oracle.prune_oracle import PruneRun
    from pyloki_gb300.config import PulsarSearchConfig

    d = load_golden(name)
    cfg = PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=False, bseg_ffa=int(d["bseg_ffa"]),
        prune_poly_order=int(d["poly_order"]), branch_max=int(d["branch_max"]),
        tiling_strategy=TILING.get(name, "aggressive"),
        p_orb_min=float(d["p_orb_min"]) if "p_orb_min" in d else 0.0)
    n = cfg.niters_ffa
    param_arr = cfg.get_param_arr(cfg.get_dparams(n))
    run = PruneRun(cfg, d["fold_ffa"], param_arr, cfg.get_dparams_actual(n), d["thresholds"],
                   max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]),
                   moving=bool(d["moving"]), nthreads=2,
                   basis=str(d["basis"]) if "basis" in d else "taylor")
    return d, run


@pytest.mark.parametrize("name", CASES)
def test_prune_oracle_matches_reference(name):
    d, run = _run(name)
    run.seed(int(d["ref_seg"]))
    np.testing.assert_array_equal(run.scheme.data, d["scheme"])
    np.testing.assert_allclose(run.leaves, d["seed_leaves"], rtol=1e-13, atol=0)
    np.testing.assert_array_equal(run.scores, d["seed_scores"])
    nparams = run.cfg.nparams
    for lvl in range(1, int(d["levels_done"]) + 1):
        assert run.step() or lvl == int(d["levels_done"])
        n_br, n_l, n_phy, n_s = run.stats[-1]
        np.testing.assert_array_equal([n_br, n_l, n_phy, n_s], d[f"stats_{lvl}"],
                                      err_msg=f"stats level {lvl}")
        np.testing.assert_array_equal(
            run.smm[-1], d[f"smm_{lvl}"].astype(np.float32).astype(np.float64),
            err_msg=f"score min/max level {lvl}")
        np.testing.assert_array_equal(run.scores, d[f"scores_{lvl}"], err_msg=f"level {lvl}")
        if f"leaves_{lvl}" in d:
            np.testing.assert_allclose(run.leaves, d[f"leaves_{lvl}"], rtol=1e-13, atol=0)
            bt = run.backtracks
            got = np.concatenate([bt[:, : nparams + 1], bt[:, -1:]], axis=1)
            np.testing.assert_array_equal(got, d[f"bt_{lvl}"], err_msg=f"bt level {lvl}")
        if f"folds_{lvl}" in d:
            np.testing.assert_array_equal(run.folds, d[f"folds_{lvl}"])
    run.ascend()
    np.testing.assert_array_equal(run.scores, d["asc_scores"])
    np.testing.assert_array_equal(run.scores_ep, d["asc_scores_ep"])
    if "asc_folds" in d:
        np.testing.assert_array_equal(run.folds, d["asc_folds"])


@pytest.mark.parametrize("tree", ["chebyshev", "circular"])
def test_prune_oracle_full_size(tree):
    """The Chebyshev oracle, and the circular-orbit oracle of order 5, over
    the pruning benchmark's series at full size (2^22 samples, 128
    segments, 127 levels, designed thresholds) against full runs of the
    reference's own Pruning (prune_large_{tree}.npz): every level's
    statistics and score range, the survivors' scores and backtracks after
    the last level, and the ascend."""
    import bench
    from oracle import oracle as O
    from oracle.prune_oracle import PruneRun

    d = load_golden(f"prune_large_{tree}")
    cfg = bench.make_prune_cfg(circular=tree == "circular")
    ts, _ = bench.make_prune_series(seed=int(d["seed"]))
    fold = O.ffa_execute(ts.ts_e, ts.ts_v, cfg)
    n = cfg.niters_ffa
    run = PruneRun(cfg, fold, cfg.get_param_arr(cfg.get_dparams(n)), cfg.get_dparams_actual(n),
                   d["thresholds"], max_sugg=bench.PRUNE_MAX_SUGG, batch_size=bench.PRUNE_BATCH,
                   basis="chebyshev" if tree == "chebyshev" else "taylor")
    run.seed(int(d["ref_seg"]))
    levels = int(d["levels_done"])
    for _ in range(levels):
        if not run.step():
            break
    np.testing.assert_array_equal(np.array(run.stats, np.int64), d["stats"])
    for lvl in range(1, levels + 1):
        np.testing.assert_array_equal(
            run.smm[lvl - 1], d[f"smm_{lvl}"].astype(np.float32).astype(np.float64),
            err_msg=f"score range level {lvl}")
    np.testing.assert_array_equal(run.scores, d["scores_last"])
    nparams = cfg.nparams
    bt = run.backtracks
    np.testing.assert_array_equal(np.concatenate([bt[:, : nparams + 1], bt[:, -1:]], axis=1),
                                  d["bt_last"])
    run.ascend()
    np.testing.assert_array_equal(run.scores, d["asc_scores"])
    np.testing.assert_array_equal(run.scores_ep, d["asc_scores_ep"])

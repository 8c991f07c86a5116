"""GPU enumerate-prune (Taylor, Chebyshev and circular-orbit trees) against
runs of the pyloki reference.

Every level is compared with the reference's tree after the same level: the
statistics, the survivor scores, the backtracks and (where stored) the folds
exactly; the FP64 leaf parameters to 1e-13 relative (they are exact on the
machine that generated the fixtures; another machine's libm pow may move the
host-computed Taylor constants by an ulp).
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ["prune_taylor", "prune_taylor_fixed", "prune_taylor_cons", "prune_taylor_quad",
         "prune_taylor_overflow", "prune_cheby", "prune_cheby_fixed", "prune_cheby_cons",
         "prune_cheby_quad", "prune_circ", "prune_circ_b4", "prune_circ_quad",
         "prune_circ_fixed"]
TILING = {"prune_taylor_cons": "conservative", "prune_taylor_quad": "quadrature",
          "prune_cheby_cons": "conservative", "prune_cheby_quad": "quadrature",
          "prune_circ_quad": "quadrature"}


def _basis(d) -> str:
    return str(d["basis"]) if "basis" in d else "taylor"


def _cfg(d, name):
    from pyloki_gb300.config import PulsarSearchConfig

    return PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=False, bseg_ffa=int(d["bseg_ffa"]),
        prune_poly_order=int(d["poly_order"]), branch_max=int(d["branch_max"]),
        tiling_strategy=TILING.get(name, "aggressive"),
        p_orb_min=float(d["p_orb_min"]) if "p_orb_min" in d else 0.0)


def _run(name, cuda_device):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = _cfg(d, name)
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device)
    dyp.initialize()
    dyp.execute()
    np.testing.assert_array_equal(dyp.fold.cpu().numpy(), d["fold_ffa"])
    prn = Pruning(dyp, d["thresholds"], max_sugg=int(d["max_sugg"]),
                  batch_size=int(d["batch_size"]), poly_basis=_basis(d),
                  use_moving_grid=bool(d["moving"]))
    return d, prn


def _leaves_close(got, ref, what, circular=False):
    if not circular:
        np.testing.assert_allclose(got, ref, rtol=1e-13, atol=0, err_msg=what)
        return
    # The circular tree: its propagation calls cos/sin, whose last bit may
    # differ between numpy and CUDA, and its secular terms cancel, so each
    # entry is compared to 1e-9 of the largest magnitude in its column.
    scale = np.abs(ref).max(axis=0, keepdims=True)
    assert np.all(np.abs(got - ref) <= 1e-9 * scale), what


@pytest.mark.parametrize("name", CASES)
def test_prune_levels_match_reference(cuda_device, name):
    d, prn = _run(name, cuda_device)
    prn.initialize(int(d["ref_seg"]))
    np.testing.assert_array_equal(prn.scheme.data, d["scheme"])
    wt = prn.world_tree
    _leaves_close(wt.leaves.cpu().numpy(), d["seed_leaves"], "seed leaves")
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d["seed_scores"])
    nparams = prn.nparams_ffa
    circ = int(d["poly_order"]) == 5
    for lvl in range(1, int(d["levels_done"]) + 1):
        prn.execute_iter()
        st = prn.pstats[-1]
        np.testing.assert_array_equal(
            [st.n_branches, st.n_leaves, st.n_leaves_phy, st.n_leaves_surv],
            d[f"stats_{lvl}"], err_msg=f"stats level {lvl}")
        np.testing.assert_array_equal([st.score_min, st.score_max],
                                      d[f"smm_{lvl}"].astype(np.float32).astype(np.float64),
                                      err_msg=f"score min/max level {lvl}")
        wt = prn.world_tree
        np.testing.assert_array_equal(wt.scores.cpu().numpy(), d[f"scores_{lvl}"],
                                      err_msg=f"scores level {lvl}")
        if f"leaves_{lvl}" in d:
            _leaves_close(wt.leaves.cpu().numpy(), d[f"leaves_{lvl}"], f"leaves level {lvl}",
                          circ)
            bt = wt.backtracks.cpu().numpy()
            got = np.concatenate([bt[:, : nparams + 1], bt[:, -1:]], axis=1)
            np.testing.assert_array_equal(got, d[f"bt_{lvl}"], err_msg=f"bt level {lvl}")
        if f"folds_{lvl}" in d:
            np.testing.assert_array_equal(wt.folds.cpu().numpy(), d[f"folds_{lvl}"])
    prn._do_ascend()
    wt = prn.world_tree
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d["asc_scores"])
    np.testing.assert_array_equal(wt.scores_ep.cpu().numpy(), d["asc_scores_ep"])
    if "asc_folds" in d:
        np.testing.assert_array_equal(wt.folds.cpu().numpy(), d["asc_folds"])
        _leaves_close(wt.leaves.cpu().numpy(), d["final_leaves"], "final leaves", circ)
        _leaves_close(prn.report(), d["report"], "report", circ)


def test_trace_integration_path(cuda_device):
    d, prn = _run("prune_taylor", cuda_device)
    prn.initialize(int(d["ref_seg"]))
    for _ in range(int(d["levels_done"])):
        prn.execute_iter()
    steps = prn.trace_integration_path(0)
    assert [s.level for s in steps] == list(range(1, len(steps) + 1))
    assert steps[-1].survivor_idx == 0
    for a, b in zip(steps[:-1], steps[1:], strict=False):
        assert b.parent_idx == a.survivor_idx
    with pytest.raises(ValueError):
        prn.trace_integration_path(10**9)


def test_prune_dyp_tree_writes_results(cuda_device, tmp_path):
    from pyloki_gb300.prune import prune_dyp_tree

    d, prn = _run("prune_taylor", cuda_device)
    from pyloki_gb300.results import LEVEL_DTYPE, read_prune_results

    path = prune_dyp_tree(prn.dyp, d["thresholds"], n_runs=2, max_sugg=int(d["max_sugg"]),
                          batch_size=int(d["batch_size"]), outdir=tmp_path, n_workers=1)
    assert path.endswith("_results.h5")
    res = read_prune_results(path)
    assert len(res["runs"]) == 2
    assert list(res["attrs"]["param_names"]) == list(prn.dyp.cfg.param_names)
    assert int(res["attrs"]["nsegments"]) == prn.dyp.nsegments
    np.testing.assert_array_equal(res["threshold_scheme"], d["thresholds"])
    for run in res["runs"].values():
        assert run["level_stats"].dtype == LEVEL_DTYPE
        assert len(run["level_stats"]) == prn.dyp.nsegments
        assert run["scores"].dtype == np.float32
        assert len(run["param_sets"]) == len(run["scores"])
    with pytest.raises(FileExistsError):
        prune_dyp_tree(prn.dyp, d["thresholds"], n_runs=2, outdir=tmp_path, n_workers=1)
    with pytest.raises(ValueError):
        prune_dyp_tree(prn.dyp, d["thresholds"], n_runs=0, outdir=tmp_path / "x")


@pytest.mark.parametrize("name", ["prune_taylor", "prune_circ"])
def test_prune_dyp_tree_drivers_match_serial(cuda_device, tmp_path, name):
    """Four runs on three worker threads and streams, and all four at once
    on the device (the default driver), write the same results as one after
    another."""
    from pyloki_gb300.prune import prune_dyp_tree

    from pyloki_gb300.results import read_prune_results

    d, prn = _run(name, cuda_device)
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]))
    a, b, c = (read_prune_results(prune_dyp_tree(prn.dyp, d["thresholds"], n_runs=4,
                                                 outdir=tmp_path / sub, **kw, **extra))
               for sub, extra in (("a", {"n_workers": 1, "driver": "threads"}),
                                  ("b", {"n_workers": 3, "driver": "threads"}),
                                  ("c", {})))
    assert list(a["runs"]) == list(b["runs"]) == list(c["runs"])
    assert len(a["runs"]) == 4
    for run in a["runs"]:
        for k in a["runs"][run]:
            np.testing.assert_array_equal(a["runs"][run][k], b["runs"][run][k], err_msg=k)
            np.testing.assert_array_equal(a["runs"][run][k], c["runs"][run][k], err_msg=k)


def test_best_intermediate_matches_get_best_k(cuda_device):
    """The per-level best leaf recorded on the device equals the host
    get_best_k of every level's tree."""
    d, prn = _run("prune_taylor", cuda_device)
    prn.initialize(int(d["ref_seg"]))
    want = []
    for _ in range(int(d["levels_done"])):
        prn.execute_iter()
        if prn.prune_complete:
            break
        want.append(prn.world_tree.get_best_k(prn.intermediate_k))
    arr = prn.best_intermediate_arr
    for lvl, (leaves, scores) in enumerate(want):
        np.testing.assert_array_equal(arr[lvl]["param_sets"], leaves)
        np.testing.assert_array_equal(arr[lvl]["scores"], scores)

"""GPU enumerate-prune against the CPU oracle and the reference on the benchmark workload.

The circular-orbit search with a Taylor tree to the 4th derivative (2^22
samples, 128 segments, FFA grid (1, 1, 1, 146)) with its designed per-level
thresholds (tests/golden/prune_scheme_taylor4.npz), run for every level from
the middle reference segment: per-level statistics, survivor scores,
backtracks and folds bit-exact, FP64 leaves to 1e-13 relative, then the
ascend. The oracle is pinned to the reference by test_prune_oracle_golden.py.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_prune_taylor4_circular_matches_oracle(cuda_device):
    import bench
    from oracle import oracle as O
    from oracle.prune_oracle import PruneRun
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning

    cfg = bench.make_prune_cfg()
    ts, _ = bench.make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=cuda_device)
    dyp.initialize()
    dyp.execute()
    fold_cpu = O.ffa_execute(ts.ts_e, ts.ts_v, cfg)
    np.testing.assert_array_equal(dyp.fold.cpu().numpy(), fold_cpu)
    nseg = dyp.nsegments
    thr = bench.prune_thresholds(nseg)
    n = cfg.niters_ffa
    run = PruneRun(cfg, fold_cpu, cfg.get_param_arr(cfg.get_dparams(n)),
                   cfg.get_dparams_actual(n), thr, max_sugg=bench.PRUNE_MAX_SUGG,
                   batch_size=bench.PRUNE_BATCH)
    prn = Pruning(dyp, thr, max_sugg=bench.PRUNE_MAX_SUGG, batch_size=bench.PRUNE_BATCH)
    ref = nseg // 2
    run.seed(ref)
    prn.initialize(ref)
    np.testing.assert_array_equal(prn.world_tree.scores.cpu().numpy(), run.scores)
    nparams = cfg.nparams
    for lvl in range(1, nseg):
        alive = run.step()
        prn.execute_iter()
        st = prn.pstats[-1]
        np.testing.assert_array_equal(
            [st.n_branches, st.n_leaves, st.n_leaves_surv],
            [run.stats[-1][0], run.stats[-1][1], run.stats[-1][3]], err_msg=f"level {lvl}")
        wt = prn.world_tree
        np.testing.assert_array_equal(wt.scores.cpu().numpy(), run.scores,
                                      err_msg=f"scores level {lvl}")
        np.testing.assert_array_equal(wt.backtracks.cpu().numpy()[:, : nparams + 1],
                                      run.backtracks[:, : nparams + 1], err_msg=f"bt {lvl}")
        np.testing.assert_array_equal(wt.backtracks.cpu().numpy()[:, -1],
                                      run.backtracks[:, -1], err_msg=f"phase bt {lvl}")
        if lvl % 16 == 0 or not alive:
            np.testing.assert_array_equal(wt.folds.cpu().numpy(), run.folds)
            np.testing.assert_allclose(wt.leaves.cpu().numpy(), run.leaves, rtol=1e-13, atol=0)
        if not alive:
            break
    assert sum(s[1] for s in run.stats) > 10**5  # the tree really branched
    prn._do_ascend()
    run.ascend()
    np.testing.assert_array_equal(prn.world_tree.scores.cpu().numpy(), run.scores)
    np.testing.assert_array_equal(prn.world_tree.folds.cpu().numpy(), run.folds)


@pytest.mark.parametrize("device_run", [False, True])
@pytest.mark.parametrize("tree", ["chebyshev", "circular"])
def test_prune_full_size_matches_reference(cuda_device, tree, device_run):
    """The same workload with the Chebyshev basis, or with the circular-orbit
    tree of order 5 (crackle added; FFA limits for order 5), against a full
    run of the reference's own Pruning (tests/golden/prune_large_{tree}.npz,
    made by make_fixtures.py --cheby-large / --circ-large from the C oracle's
    FFA fold of the same seeded series): every level's statistics and score
    range, the surviving scores and backtracks after the last level, the
    ascend and the report (the circular tree's to 1e-9 of each column's
    largest magnitude: its propagation calls cos/sin)."""
    import bench
    from conftest import load_golden
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning
    from tests.test_prune_gpu import _leaves_close

    d = load_golden(f"prune_large_{tree}")
    circ = tree == "circular"
    cfg = bench.make_prune_cfg(circular=circ)
    ts, _ = bench.make_prune_series(seed=int(d["seed"]))
    dyp = DynamicProgramming(ts, cfg, device=cuda_device)
    dyp.initialize()
    dyp.execute()
    prn = Pruning(dyp, d["thresholds"], max_sugg=bench.PRUNE_MAX_SUGG,
                  batch_size=bench.PRUNE_BATCH, poly_basis="taylor" if circ else tree)
    assert prn.circular == circ
    ref = int(d["ref_seg"])
    levels = int(d["levels_done"])
    if device_run:
        prn.run_device(ref, graph=True, levels=levels)
    else:
        prn.initialize(ref)
        for _ in range(levels):
            prn.execute_iter()
    got = np.array([[s.n_branches, s.n_leaves, s.n_leaves_phy, s.n_leaves_surv]
                    for s in prn.pstats[1:]], np.int64)
    np.testing.assert_array_equal(got, d["stats"])
    for lvl in range(1, levels + 1):
        st = prn.pstats[lvl]
        np.testing.assert_array_equal([st.score_min, st.score_max],
                                      d[f"smm_{lvl}"].astype(np.float32).astype(np.float64),
                                      err_msg=f"score range level {lvl}")
    wt = prn.world_tree
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d["scores_last"])
    nparams = cfg.nparams
    bt = wt.backtracks.cpu().numpy()
    np.testing.assert_array_equal(np.concatenate([bt[:, : nparams + 1], bt[:, -1:]], axis=1),
                                  d["bt_last"])
    prn._do_ascend()
    wt = prn.world_tree
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d["asc_scores"])
    np.testing.assert_array_equal(wt.scores_ep.cpu().numpy(), d["asc_scores_ep"])
    if circ:
        _leaves_close(prn.report(), d["report"], "report", circular=True)
    else:
        np.testing.assert_allclose(prn.report(), d["report"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("tree", ["chebyshev", "circular"])
def test_prune_full_size_matches_oracle(cuda_device, tree):
    """The Chebyshev tree, and the circular-orbit tree of order 5, on the
    benchmark workload level by level against the C oracle (itself pinned
    to the reference's full runs by test_prune_oracle_golden.py): every
    level's statistics, survivor scores and backtracks, the folds and
    leaves every 16 levels and at the end, then the ascend."""
    import bench
    from oracle import oracle as O
    from oracle.prune_oracle import PruneRun
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning
    from tests.test_prune_gpu import _leaves_close

    circ = tree == "circular"
    cfg = bench.make_prune_cfg(circular=circ)
    ts, _ = bench.make_prune_series(seed=2000)
    dyp = DynamicProgramming(ts, cfg, device=cuda_device)
    dyp.initialize()
    dyp.execute()
    fold_cpu = O.ffa_execute(ts.ts_e, ts.ts_v, cfg)
    np.testing.assert_array_equal(dyp.fold.cpu().numpy(), fold_cpu)
    nseg = dyp.nsegments
    thr = bench.prune_thresholds(nseg)
    n = cfg.niters_ffa
    basis = "taylor" if circ else "chebyshev"
    run = PruneRun(cfg, fold_cpu, cfg.get_param_arr(cfg.get_dparams(n)),
                   cfg.get_dparams_actual(n), thr, max_sugg=bench.PRUNE_MAX_SUGG,
                   batch_size=bench.PRUNE_BATCH, basis=basis)
    prn = Pruning(dyp, thr, max_sugg=bench.PRUNE_MAX_SUGG, batch_size=bench.PRUNE_BATCH,
                  poly_basis=basis)
    ref = nseg // 2
    run.seed(ref)
    prn.initialize(ref)
    np.testing.assert_array_equal(prn.world_tree.scores.cpu().numpy(), run.scores)
    nparams = cfg.nparams
    for lvl in range(1, nseg):
        alive = run.step()
        prn.execute_iter()
        st = prn.pstats[-1]
        np.testing.assert_array_equal(
            [st.n_branches, st.n_leaves, st.n_leaves_phy, st.n_leaves_surv],
            list(run.stats[-1]), err_msg=f"level {lvl}")
        wt = prn.world_tree
        np.testing.assert_array_equal(wt.scores.cpu().numpy(), run.scores,
                                      err_msg=f"scores level {lvl}")
        bt = wt.backtracks.cpu().numpy()
        np.testing.assert_array_equal(bt[:, : nparams + 1], run.backtracks[:, : nparams + 1],
                                      err_msg=f"bt {lvl}")
        np.testing.assert_array_equal(bt[:, -1], run.backtracks[:, -1], err_msg=f"phase {lvl}")
        if lvl % 16 == 0 or not alive:
            np.testing.assert_array_equal(wt.folds.cpu().numpy(), run.folds)
            _leaves_close(wt.leaves.cpu().numpy(), run.leaves, f"leaves {lvl}", circ)
        if not alive:
            break
    prn._do_ascend()
    run.ascend()
    np.testing.assert_array_equal(prn.world_tree.scores.cpu().numpy(), run.scores)
    np.testing.assert_array_equal(prn.world_tree.folds.cpu().numpy(), run.folds)

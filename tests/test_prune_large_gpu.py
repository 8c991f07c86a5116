"""GPU enumerate-prune against the CPU oracle on the benchmark workload.

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

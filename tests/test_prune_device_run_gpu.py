"""Device-resident pruning runs (loki_prune_run) against the reference and
against the level-by-level path.

``Pruning.run_device`` enqueues every level of a reference segment with the
counts kept on the device; the level statistics, the surviving tree, the
per-level backtracks and best leaves, and the ascend that follows must equal
the reference's runs (the same fixtures as test_prune_gpu.py) and the
level-by-level path, with and without CUDA-graph capture and replay.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.test_prune_gpu import _leaves_close, _run

pytestmark = pytest.mark.gpu
CASES = ["prune_taylor", "prune_taylor_fixed", "prune_taylor_cons", "prune_taylor_quad",
         "prune_taylor_overflow", "prune_cheby", "prune_cheby_fixed", "prune_cheby_cons",
         "prune_cheby_quad", "prune_circ", "prune_circ_b4", "prune_circ_quad",
         "prune_circ_fixed"]


def _check_against_fixture(d, prn, levels):
    circ = int(d["poly_order"]) == 5
    for lvl in range(1, levels + 1):
        if lvl >= len(prn.pstats):
            break
        st = prn.pstats[lvl]
        np.testing.assert_array_equal(
            [st.n_branches, st.n_leaves, st.n_leaves_phy, st.n_leaves_surv],
            d[f"stats_{lvl}"], err_msg=f"stats level {lvl}")
        np.testing.assert_array_equal([st.score_min, st.score_max],
                                      d[f"smm_{lvl}"].astype(np.float32).astype(np.float64),
                                      err_msg=f"score min/max level {lvl}")
    last = prn.prune_level
    wt = prn.world_tree
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d[f"scores_{last}"])
    if f"leaves_{last}" in d:
        _leaves_close(wt.leaves.cpu().numpy(), d[f"leaves_{last}"], "final leaves", circ)
    if f"folds_{last}" in d:
        np.testing.assert_array_equal(wt.folds.cpu().numpy(), d[f"folds_{last}"])
    prn._do_ascend()
    wt = prn.world_tree
    np.testing.assert_array_equal(wt.scores.cpu().numpy(), d["asc_scores"])
    np.testing.assert_array_equal(wt.scores_ep.cpu().numpy(), d["asc_scores_ep"])
    if "asc_folds" in d:
        np.testing.assert_array_equal(wt.folds.cpu().numpy(), d["asc_folds"])
        _leaves_close(wt.leaves.cpu().numpy(), d["final_leaves"], "ascended leaves", circ)
        _leaves_close(prn.report(), d["report"], "report", circ)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", CASES)
def test_device_run_matches_reference(cuda_device, name, graph):
    d, prn = _run(name, cuda_device)
    levels = int(d["levels_done"])
    ref = int(d["ref_seg"])
    for _ in range(2):  # the second run replays the captured graph
        prn.run_device(ref, graph=graph, levels=levels)
        np.testing.assert_array_equal(prn.scheme.data, d["scheme"])
        _check_against_fixture(d, prn, levels)


@pytest.mark.parametrize("name", ["prune_taylor", "prune_taylor_overflow", "prune_cheby",
                                  "prune_circ", "prune_circ_b4"])
def test_device_run_matches_level_path(cuda_device, name):
    """Backtrack history, per-level best leaves and statistics equal the
    level-by-level path's."""
    d, prn = _run(name, cuda_device)
    levels = int(d["levels_done"])
    ref = int(d["ref_seg"])
    prn.initialize(ref)
    for _ in range(levels):
        prn.execute_iter()
    want_stats = [(s.n_branches, s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
                  for s in prn.pstats]
    want_bt = [b.cpu().numpy() for b in prn.backtrack_hist]
    want_best = prn.best_intermediate_arr.copy()
    want_tree = prn.world_tree.leaves.cpu().numpy()
    prn.run_device(ref, graph=True, levels=levels)
    got_stats = [(s.n_branches, s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
                 for s in prn.pstats]
    assert got_stats == want_stats
    got_bt = [b.cpu().numpy() for b in prn.backtrack_hist]
    assert len(got_bt) == len(want_bt)
    for lvl, (a, b) in enumerate(zip(got_bt, want_bt, strict=True)):
        np.testing.assert_array_equal(a, b, err_msg=f"backtracks level {lvl + 1}")
    got_best = prn.best_intermediate_arr
    np.testing.assert_array_equal(got_best["scores"], want_best["scores"])
    np.testing.assert_array_equal(got_best["param_sets"], want_best["param_sets"])
    np.testing.assert_array_equal(prn.world_tree.leaves.cpu().numpy(), want_tree)


@pytest.mark.parametrize("name", ["prune_taylor", "prune_circ"])
def test_device_run_grows_its_workspace(cuda_device, name):
    """A child workspace that is too small is detected on the device, grown
    and the run repeated: the results do not change."""
    d, prn = _run(name, cuda_device)
    levels = int(d["levels_done"])
    ref = int(d["ref_seg"])
    prn.device_child_cap = 64
    prn.run_device(ref, levels=levels)
    assert max(s.n_leaves for s in prn.pstats[1:]) > 64
    assert prn._device_bufs.child_cap > 64
    _check_against_fixture(d, prn, levels)


def test_device_run_rejects_unsupported(cuda_device):
    """A parent hook or more than one best leaf per level stays on the
    level-by-level path."""
    from pyloki_gb300.prune import Pruning

    d, prn = _run("prune_circ", cuda_device)
    assert prn.device_run_supported
    prn.parent_hook = lambda p, tree, level: None
    assert not prn.device_run_supported
    with pytest.raises(ValueError):
        prn.run_device(int(d["ref_seg"]))
    p2 = Pruning(prn.dyp, d["thresholds"], max_sugg=int(d["max_sugg"]),
                 batch_size=int(d["batch_size"]), intermediate_k=2)
    assert not p2.device_run_supported


@pytest.mark.parametrize("n_streams", [1, 3])
def test_run_batch_matches_level_path(cuda_device, n_streams):
    """Batched device-resident runs of several reference segments (one graph
    per run, runs on concurrent streams) equal level-by-level runs."""
    from pyloki_gb300.prune import Pruning, run_batch

    d, prn = _run("prune_taylor", cuda_device)
    dyp = prn.dyp
    refs = [0, 3, 7, dyp.nsegments - 1, 5]
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]))
    got = run_batch([(dyp, r) for r in refs], d["thresholds"], n_streams=n_streams, **kw)
    again = run_batch([(dyp, r) for r in refs], d["thresholds"], n_streams=n_streams, **kw)
    for ref, g, a in zip(refs, got, again, strict=True):
        p = Pruning(dyp, d["thresholds"], **kw)
        p.initialize(ref)
        for _ in range(dyp.nsegments - 1):
            p.execute_iter()
        p._do_ascend()
        want_stats = [(s.n_branches, s.n_leaves, s.n_leaves_surv) for s in p.pstats]
        for res in (g, a):
            assert [(s.n_branches, s.n_leaves, s.n_leaves_surv)
                    for s in res["level_stats"]] == want_stats
            np.testing.assert_array_equal(res["scores"], p.world_tree.scores.cpu().numpy())
            np.testing.assert_array_equal(res["scores_ep"],
                                          p.world_tree.scores_ep.cpu().numpy())
            np.testing.assert_array_equal(res["param_sets"], p.report())


def test_prune_batch_rebinds_to_new_folds(cuda_device):
    """A PruneBatch keeps its graphs across folds of the same configuration:
    runs over a second series (the first one's noise reversed) equal the
    level-by-level runs of that series."""
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBatch, Pruning
    from pyloki_gb300.timeseries import TimeSeries

    d, prn = _run("prune_taylor", cuda_device)
    cfg = prn.dyp.cfg
    dyp2 = DynamicProgramming(TimeSeries(d["ts_e"][::-1].copy(), d["ts_v"], cfg.tsamp), cfg,
                              device=cuda_device)
    dyp2.initialize()
    dyp2.execute()
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]))
    runner = PruneBatch(d["thresholds"], n_streams=2, **kw)
    refs = [1, 6, 9]
    for dyp in (prn.dyp, dyp2, prn.dyp, dyp2):
        got = runner.run([(dyp, r) for r in refs])
        for ref, g in zip(refs, got, strict=True):
            p = Pruning(dyp, d["thresholds"], **kw)
            p.initialize(ref)
            for _ in range(dyp.nsegments - 1):
                p.execute_iter()
            p._do_ascend()
            assert [(s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
                    for s in g["level_stats"]] == [
                (s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max) for s in p.pstats]
            np.testing.assert_array_equal(g["scores"], p.world_tree.scores.cpu().numpy())
            np.testing.assert_array_equal(g["param_sets"], p.report())


def _level_path_results(prn_factory, dyp, ref, d):
    p = prn_factory()
    p.initialize(ref)
    for _ in range(dyp.nsegments - 1):
        p.execute_iter()
    p._do_ascend()
    return ([(s.n_branches, s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
             for s in p.pstats], p.world_tree.scores.cpu().numpy(),
            p.world_tree.scores_ep.cpu().numpy(), p.report())


@pytest.mark.parametrize("name", ["prune_taylor", "prune_taylor_overflow", "prune_cheby",
                                  "prune_taylor_quad", "prune_cheby_fixed", "prune_circ",
                                  "prune_circ_b4"])
@pytest.mark.parametrize("max_jobs", [3, 64])
@pytest.mark.parametrize("driver", ["batch", "blocks"])
def test_block_batch_matches_level_path(cuda_device, name, max_jobs, driver):
    """The level-synchronous batch (loki_prune_batch_*) and one thread block
    per job (loki_prune_run_blocks): every job's level records, final scores,
    ascend and report equal the level-by-level run's, in one launch or in
    waves of three; the overflow fixture runs the overflow rule, the
    circular-orbit fixtures (batch of 64 and of 4 parents) the circular
    level's child map, validity compaction and batch offsets."""
    from pyloki_gb300.prune import PruneBlockBatch, Pruning

    d, prn = _run(name, cuda_device)
    dyp = prn.dyp
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]),
              poly_basis=prn.poly_basis, use_moving_grid=prn.use_moving_grid)
    refs = [0, 3, int(d["ref_seg"]), dyp.nsegments - 1, 5, 9, 12]
    runner = PruneBlockBatch(d["thresholds"], max_jobs=max_jobs, driver=driver, **kw)
    # the second call reuses the slots' buffers and runs; with the batch
    # driver it captures the kernels in a CUDA graph, which the third replays
    for _ in range(3):
        got = runner.run([(dyp, r) for r in refs])
        for ref, g in zip(refs, got, strict=True):
            want = _level_path_results(lambda: Pruning(dyp, d["thresholds"], **kw), dyp, ref, d)
            assert [(s.n_branches, s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
                    for s in g["level_stats"]] == want[0], ref
            np.testing.assert_array_equal(g["scores"], want[1])
            np.testing.assert_array_equal(g["scores_ep"], want[2])
            np.testing.assert_array_equal(g["param_sets"], want[3])


@pytest.mark.parametrize(("name", "driver"), [("prune_taylor", "batch"),
                                             ("prune_taylor", "blocks"),
                                             ("prune_circ", "batch")])
def test_block_batch_grows_workspaces(cuda_device, name, driver):
    """A job whose children outgrow the batched drivers' workspace is flagged
    on the device and repeated with grown buffers: the results do not change."""
    from pyloki_gb300.prune import PruneBlockBatch, Pruning

    d, prn = _run(name, cuda_device)
    dyp = prn.dyp
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]))
    runner = PruneBlockBatch(d["thresholds"], max_jobs=4, driver=driver, **kw)
    for k in range(2):
        runner._slot(k, dyp).device_child_cap = 64
    refs = [int(d["ref_seg"]), 2]
    got = runner.run([(dyp, r) for r in refs])
    for ref, g in zip(refs, got, strict=True):
        want = _level_path_results(lambda: Pruning(dyp, d["thresholds"], **kw), dyp, ref, d)
        assert max(s.n_leaves for s in g["level_stats"]) > 64
        np.testing.assert_array_equal(g["scores"], want[1])
        np.testing.assert_array_equal(g["param_sets"], want[3])


def test_block_batch_passes_circular_to_streams(cuda_device):
    """The block-per-run driver hands circular-orbit trees to PruneBatch."""
    from pyloki_gb300.prune import PruneBlockBatch, run_batch

    d, prn = _run("prune_circ", cuda_device)
    dyp = prn.dyp
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]))
    refs = [int(d["ref_seg"]), 1]
    got = PruneBlockBatch(d["thresholds"], driver="blocks", **kw).run([(dyp, r) for r in refs])
    want = run_batch([(dyp, r) for r in refs], d["thresholds"], n_streams=2, **kw)
    for g, w in zip(got, want, strict=True):
        np.testing.assert_array_equal(g["scores"], w["scores"])
        np.testing.assert_array_equal(g["param_sets"], w["param_sets"])


@pytest.mark.parametrize("name", ["prune_taylor_fourier", "prune_cheby_fourier",
                                  "prune_circ_fourier"])
def test_block_batch_fourier_matches_level_path(cuda_device, name):
    """Complex (Fourier-domain) trees in the level-synchronous batch: every
    job's level records, final scores, ascend and report equal the
    level-by-level complex run's, uncaptured, captured and replayed, and
    with a workspace too small for some levels (repeated through the batch
    with grown buffers); the block-per-run driver declines them."""
    from pyloki_gb300.config import PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import PruneBlockBatch, Pruning
    from pyloki_gb300.timeseries import TimeSeries
    from tests.conftest import load_golden

    d = load_golden(name)
    cfg = PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=True, bseg_ffa=int(d["bseg_ffa"]),
        prune_poly_order=int(d["poly_order"]), branch_max=int(d["branch_max"]),
        p_orb_min=float(d["p_orb_min"]))
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device)
    dyp.initialize()
    dyp.execute()
    basis = str(d["basis"]) if "basis" in d else "taylor"
    kw = dict(max_sugg=int(d["max_sugg"]), batch_size=int(d["batch_size"]), poly_basis=basis,
              use_moving_grid=bool(d["moving"]))
    assert Pruning(dyp, d["thresholds"], **kw).fourier
    refs = [0, int(d["ref_seg"]), dyp.nsegments - 1, 6]
    runner = PruneBlockBatch(d["thresholds"], **kw)
    for _ in range(3):
        got = runner.run([(dyp, r) for r in refs])
        for ref, g in zip(refs, got, strict=True):
            want = _level_path_results(lambda: Pruning(dyp, d["thresholds"], **kw), dyp, ref, d)
            assert [(s.n_branches, s.n_leaves, s.n_leaves_surv, s.score_min, s.score_max)
                    for s in g["level_stats"]] == want[0], ref
            np.testing.assert_array_equal(g["scores"], want[1])
            np.testing.assert_array_equal(g["scores_ep"], want[2])
            np.testing.assert_array_equal(g["param_sets"], want[3])
    small = PruneBlockBatch(d["thresholds"], max_jobs=4, **kw)
    for k in range(2):
        small._slot(k, dyp).device_child_cap = 64
    got = small.run([(dyp, r) for r in refs[:2]])
    for ref, g in zip(refs[:2], got, strict=True):
        want = _level_path_results(lambda: Pruning(dyp, d["thresholds"], **kw), dyp, ref, d)
        assert max(s.n_leaves for s in g["level_stats"]) > 64
        np.testing.assert_array_equal(g["scores"], want[1])
        np.testing.assert_array_equal(g["param_sets"], want[3])
    with pytest.raises(ValueError, match="driver='batch'"):
        PruneBlockBatch(d["thresholds"], driver="blocks", **kw).run([(dyp, refs[0])])

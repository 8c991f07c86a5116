"""Learned branch proposal on the GPU: the parent hook leaves plain pruning
unchanged when it keeps every parent; under a budget every emitted leaf still
passes the exact threshold and is a leaf the plain run also emits; and the
training study runs end to end on the circular-orbit Taylor workload."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NSAMPS = 2**20


def _cfg():
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig

    lim = ParamLimits.from_circular(333.33, p_orb_min=7200.0, poly_order=4)
    return PulsarSearchConfig(nsamps=NSAMPS, tsamp=64e-6, nbins=64, eta=1.0,
                              param_limits=lim.limits, use_fourier=False, bseg_ffa=NSAMPS // 32,
                              prune_poly_order=4)


def _series(seed, inject=True):
    from pyloki_gb300.simulation import make_series

    rng = np.random.default_rng(seed)
    orbit = (rng.uniform(2.0, 10.0) * 3600.0, rng.uniform(0.1, 2.0), rng.uniform(0, 2 * np.pi))
    if not inject:
        return make_series(NSAMPS, 64e-6, seed=seed)
    return make_series(NSAMPS, 64e-6, freq=333.33, snr=12.0, orbit=orbit, seed=seed)


def _run(cfg, ts, hook, dev, max_sugg=2**16):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning

    d = DynamicProgramming(ts, cfg, device=dev)
    d.initialize()
    d.execute()
    thr = 4.0 * np.sqrt(np.arange(1, d.nsegments) / (d.nsegments - 1))
    prn = Pruning(d, thr, max_sugg=max_sugg)
    prn.parent_hook = hook
    prn.initialize(d.nsegments // 2)
    for _ in range(d.nsegments - 1):
        prn.execute_iter()
        if prn.prune_complete:
            break
    return prn, thr


def test_hook_that_keeps_all_parents_is_plain(cuda_device):
    from pyloki_gb300.learned import Recorder

    cfg, ts = _cfg(), _series(5)
    a, _ = _run(cfg, ts, None, cuda_device)
    rec = Recorder(per_level=256)
    b, _ = _run(cfg, ts, rec, cuda_device)
    assert [s.n_leaves for s in a.pstats] == [s.n_leaves for s in b.pstats]
    np.testing.assert_array_equal(a.world_tree.leaves.cpu().numpy(),
                                  b.world_tree.leaves.cpu().numpy())
    np.testing.assert_array_equal(a.world_tree.scores.cpu().numpy(),
                                  b.world_tree.scores.cpu().numpy())
    x, y = rec.labels(b, lookahead=4)
    assert x.shape[1] == 16 and x.shape[0] == y.shape[0] > 0
    assert 0.0 < float(y.mean()) <= 1.0


def test_budget_keeps_exact_threshold_and_plain_leaves(cuda_device):
    from pyloki_gb300.learned import BranchMLP, BranchProposal

    cfg, ts = _cfg(), _series(6)
    plain, thr = _run(cfg, ts, None, cuda_device)
    sizes = [s.n_branches for s in plain.pstats[1:]]
    budget = max(8, int(np.median(sizes)) // 2)
    prop = BranchProposal(BranchMLP(device=cuda_device, seed=3), budget)
    got, _ = _run(cfg, ts, prop, cuda_device)
    assert prop.levels_cut > 0 and got.parents_skipped > 0
    # ties at the cut may keep a few more than the budget
    assert all(s.n_branches <= budget + 64 for s in got.pstats[1:])
    wt = got.world_tree
    if wt.valid_size:
        level = got.prune_level
        assert float(wt.scores.min()) >= thr[level - 1]
        # every learned leaf is a leaf of the plain run (same parents, same
        # children, same exact threshold)
        if plain.prune_level == level:
            pl = {r.tobytes() for r in plain.world_tree.leaves.cpu().numpy()}
            assert all(r.tobytes() in pl for r in wt.leaves.cpu().numpy())
    # backtracks point into the full (unrestricted) parent tree of each level
    for k, bt in enumerate(got.backtrack_hist):
        assert 0 <= int(bt[:, 0].min()) and int(bt[:, 0].max()) < got.pstats[k].n_leaves_surv


def test_study_runs_end_to_end(cuda_device):
    from pyloki_gb300.learned import study

    cfg = _cfg()
    res = study(cfg, 4.0 * np.sqrt(np.arange(1, 32) / 31), _series, train_seeds=[11, 12],
                test_seeds=[21], noise_seeds=[31], budget=2048, lookahead=4, per_level=512,
                epochs=2, max_sugg=2**16, device=cuda_device)
    assert res["train_samples"] > 0 and len(res["loss_per_epoch"]) == 2
    b = res["budgets"]["2048"]
    assert 0.0 <= b["recall_vs_plain"] <= 1.0
    assert res["plain_leaves_per_s"] > 0 and b["learned_leaves_per_s"] > 0
    assert b["leaves_fraction"] <= 1.0


def test_trained_network_beats_untrained_at_equal_budget(cuda_device):
    """What training buys: at the same parent budget, a network trained on
    plain runs keeps more of the plain run's best final leaves (held-out
    injections) than the same network before training."""
    from pyloki_gb300.learned import BranchMLP, BranchProposal, Recorder

    cfg = _cfg()
    xs, ys = [], []
    for sd in (41, 42, 43, 44, 45, 46):
        rec = Recorder(per_level=1024, seed=sd)
        prn, _ = _run(cfg, _series(sd), rec, cuda_device)
        x, y = rec.labels(prn, lookahead=4, top_k=16)
        xs.append(x)
        ys.append(y)
    x, y = torch.cat(xs), torch.cat(ys)
    pos = float(y.mean())
    wt = torch.where(y > 0.5, 0.5 / pos, 0.5 / (1 - pos))
    trained = BranchMLP(device=cuda_device, seed=5)
    trained.fit(x, y, wt, epochs=6, batch=4096, lr=2e-3)
    untrained = BranchMLP(device=cuda_device, seed=5)

    def recovered(net, sd, budget):
        plain, _ = _run(cfg, _series(sd), None, cuda_device)
        wt0 = plain.world_tree
        top = torch.topk(wt0.scores, min(16, wt0.valid_size)).indices
        want = {r.tobytes() for r in wt0.leaves[top].cpu().numpy()}
        got, _ = _run(cfg, _series(sd), BranchProposal(net, budget), cuda_device)
        have = {r.tobytes() for r in got.world_tree.leaves.cpu().numpy()}
        return len(want & have) / max(len(want), 1)

    plain, _ = _run(cfg, _series(61), None, cuda_device)
    budget = max(64, int(np.median([s.n_branches for s in plain.pstats[1:]])) // 4)
    rec_t = [recovered(trained, sd, budget) for sd in (61, 62, 63, 64)]
    rec_u = [recovered(untrained, sd, budget) for sd in (61, 62, 63, 64)]
    print(f"budget {budget}: recovered top-16 trained {rec_t} untrained {rec_u}")
    assert np.mean(rec_t) > np.mean(rec_u), (rec_t, rec_u)

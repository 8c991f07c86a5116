"""Host logic of the batched pruning drivers that needs no GPU: the level
records of a device run read back into ``PruneStats`` (the reference's
per-level statistics, ``io/cands.py:17-103``), the last level and survivor
count of a run, and the reuse of the level tables across calls."""

from __future__ import annotations

import ctypes as C
import types

import numpy as np
import pytest
import torch

from pyloki_gb300 import _lib
from pyloki_gb300.prune import PruneBlockBatch, PruneStats, _DeviceRun


def _run_with_stats(nlev: int, seed_n: int, stats: np.ndarray) -> _DeviceRun:
    dr = _DeviceRun.__new__(_DeviceRun)  # the host half only: no buffers, no GPU
    dr.nlev = nlev
    dr.scheme = types.SimpleNamespace(get_segment_idx=lambda i: 7)
    dr.seed = types.SimpleNamespace(size=seed_n)
    dr._h_seed = torch.arange(1.0, seed_n + 1.0)
    dr._h_stats = torch.from_numpy(stats.view(np.uint8).copy())
    dr._h_err = torch.zeros(1, dtype=torch.int32)
    dr.seg_idx = np.arange(nlev, dtype=np.int32)
    dr.thresholds = np.linspace(0, 4, nlev)
    return dr


def _records(nlev: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    st = np.zeros(nlev, _lib.PRUNE_STATS_DTYPE)
    for k in ("n_parents", "n_children", "n_valid", "n_surv"):
        st[k] = rng.integers(1, 1000, nlev)
    st["n_children"][::7] = 0
    st["score_min"] = rng.random(nlev)
    st["score_max"] = rng.random(nlev) + 1
    return st


@pytest.mark.parametrize("dead_at", [None, 1, 5, 127])
def test_stats_host_stops_at_the_first_empty_level(dead_at):
    """(records, error word, last level, survivors of it): the run ends at
    its first level without survivors, else at its last level."""
    nlev = 127
    st = _records(nlev, 1)
    if dead_at is not None:
        st["n_surv"][dead_at - 1] = 0
        st["n_surv"][dead_at:] = 0
    _, err, last, n_final = _run_with_stats(nlev, 3, st).stats_host()
    assert err == 0
    want_last = dead_at if dead_at is not None else nlev
    assert last == want_last
    assert n_final == int(st["n_surv"][want_last - 1])
    assert _run_with_stats(0, 3, st).stats_host()[2:] == (0, 3)  # no level: the seed


@pytest.mark.parametrize("last", [0, 1, 5, 127])
def test_level_stats_match_the_records(last):
    """PruneStats of level 0 (the seed) and of every level up to ``last``,
    field by field, with no score range on a level without children."""
    nlev = 127
    st = _records(nlev, 2)
    dr = _run_with_stats(nlev, 3, st)
    got = dr.level_stats(st, last)
    assert got[0] == PruneStats(level=0, seg_idx=7, threshold=0, score_min=1.0, score_max=3.0,
                                n_branches=3, n_leaves=3, n_leaves_phy=3, n_leaves_surv=3)
    f = st[:last]
    want = [PruneStats(level=i + 1, seg_idx=i, threshold=float(dr.thresholds[i]),
                       score_min=float(f["score_min"][i]) if f["n_children"][i] else 0.0,
                       score_max=float(f["score_max"][i]) if f["n_children"][i] else 0.0,
                       n_branches=int(f["n_parents"][i]), n_leaves=int(f["n_children"][i]),
                       n_leaves_phy=int(f["n_valid"][i]), n_leaves_surv=int(f["n_surv"][i]))
            for i in range(last)]
    assert got[1:] == want
    assert all(type(s.n_leaves) is int and type(s.score_max) is float for s in got[1:])


def _fake_run(ref: int, nlev: int):
    dr = types.SimpleNamespace(ref_seg=ref, nlev=nlev)
    dr.descs = (_lib.LokiPruneLevel * nlev)()
    for i in range(nlev):
        dr.descs[i].nbins = 1000 * ref + i  # a recognisable field per (run, level)
    dr.seg_idx = np.arange(nlev, dtype=np.int32) + ref
    dr.thresholds = np.full(nlev, float(ref))
    return dr


def test_level_tables_are_kept_while_the_runs_are_unchanged(monkeypatch):
    """The level descriptors, segment order and thresholds of a batch are
    laid out job after job, reused while the same runs come back, and laid
    out again when a run changes."""
    pinned = []

    def fake_empty(n, dtype, pin_memory=False):  # pinned memory needs a GPU
        t = torch.zeros(n, dtype=dtype)
        pinned.append(pin_memory)
        return t

    monkeypatch.setattr(torch, "empty", fake_empty)
    b = PruneBlockBatch.__new__(PruneBlockBatch)
    prn = object()
    runs = [(prn, _fake_run(r, 4)) for r in (3, 8, 5)]
    lv, seg, thr = b._level_tables(runs, 4)
    assert pinned == [True]
    assert [lv[i].nbins for i in range(12)] == [1000 * r + i for r in (3, 8, 5) for i in range(4)]
    np.testing.assert_array_equal(seg[1], np.arange(4) + 8)
    np.testing.assert_array_equal(thr[:, 0], [3.0, 8.0, 5.0])
    assert b._level_tables(runs, 4)[0] is lv  # the same runs: kept
    runs[1] = (prn, _fake_run(9, 4))
    lv2, seg2, _ = b._level_tables(runs, 4)
    assert lv2[4].nbins == 9000 and seg2[1, 0] == 9
    assert C.sizeof(lv2) == 12 * C.sizeof(_lib.LokiPruneLevel)

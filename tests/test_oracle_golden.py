"""The C oracle against fixtures produced by the pyloki reference itself."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import cfg_from_golden, load_golden

FFA_CASES = ["ffa_freq", "ffa_accel", "ffa_jerk"]
SCORE_CASES = ["score_nb64", "score_nb50", "score_nb100"]


@pytest.mark.parametrize("name", FFA_CASES)
def test_oracle_ffa_levels_bit_exact(name):
    d = load_golden(name)
    cfg = cfg_from_golden(d)
    levels = O.ffa_execute(d["ts_e"], d["ts_v"], cfg, nthreads=2, keep_levels=True)
    assert len(levels) == int(d["niters"]) + 1
    for lvl, fold in enumerate(levels):
        ref = d[f"fold_{lvl}"]
        assert fold.shape == ref.shape
        np.testing.assert_array_equal(fold, ref, err_msg=f"level {lvl}")


@pytest.mark.parametrize("name", FFA_CASES)
def test_oracle_plan_matches_reference_resolve(name):
    d = load_golden(name)
    cfg = cfg_from_golden(d)
    for lvl in range(1, cfg.niters_ffa + 1):
        it, pt, ih, ph = O.ffa_plan(cfg, lvl, nthreads=2)
        np.testing.assert_array_equal(it, d[f"plan_i_tail_{lvl}"])
        np.testing.assert_array_equal(ih, d[f"plan_i_head_{lvl}"])
        np.testing.assert_array_equal(pt, d[f"plan_shift_tail_{lvl}"])
        np.testing.assert_array_equal(ph, d[f"plan_shift_head_{lvl}"])


def test_oracle_plan_freq_matches_ffaplan():
    d = load_golden("ffa_freq")
    cfg = cfg_from_golden(d)
    for lvl in range(1, cfg.niters_ffa + 1):
        _, _, ih, ph = O.ffa_plan(cfg, lvl)
        np.testing.assert_array_equal(ih.astype(np.uint32), d[f"plan_idx_{lvl}"])
        np.testing.assert_array_equal(ph.astype(np.float32), d[f"plan_shift_{lvl}"])


@pytest.mark.parametrize("name", FFA_CASES)
def test_oracle_norm_and_snr(name):
    d = load_golden(name)
    fn = O.fold_norm(d[f"fold_{int(d['niters'])}"][0])
    np.testing.assert_array_equal(fn, d["fold_norm"])
    np.testing.assert_array_equal(O.boxcar_snr(fn, d["widths"]), d["snrs"])


@pytest.mark.parametrize("name", SCORE_CASES)
def test_oracle_scoring(name):
    d = load_golden(name)
    np.testing.assert_array_equal(O.boxcar_snr(d["prof"], d["widths"]), d["snr"])
    np.testing.assert_array_equal(O.boxcar_snr(d["prof"], d["widths"], 1.7), d["snr_std"])
    np.testing.assert_array_equal(O.snr_score_batch(d["comb"], d["widths"]), d["score"])


def test_oracle_detects_planted_error():
    """A mistake planted in the oracle's input must be caught by the comparison."""
    d = load_golden("ffa_freq")
    cfg = cfg_from_golden(d)
    ts_e = d["ts_e"].copy()
    ts_e[123] += 1.0
    fold = O.ffa_initialize(ts_e, d["ts_v"], cfg)
    assert not np.array_equal(fold, d["fold_0"])

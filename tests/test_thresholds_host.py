"""Threshold-scheme design, host side (CPU): the profile template, the
reference's bound and trials schemes, state transitions and beam neighbours."""

from __future__ import annotations

import numpy as np
from scipy import stats

from pyloki_gb300.thresholds import (bound_scheme, generate_folded_profile, get_next_state,
                                     initial_state, neighbouring_indices, state_dtype,
                                     trials_scheme)


def test_folded_profile_is_unit_norm_gaussian_centred():
    p = generate_folded_profile(nbins=64, ducy=0.1)
    assert abs(np.sum(p**2) - 1.0) < 1e-12
    assert int(np.argmax(p)) == 32
    np.testing.assert_allclose(p[31], p[33])


def test_bound_and_trials_schemes():
    b = bound_scheme(9, 8.0)
    assert len(b) == 9
    np.testing.assert_allclose(b**2, np.arange(2, 11) * 64.0 / 10, rtol=1e-6)
    bp = np.array([2.0, 3.0, 2.0])
    np.testing.assert_allclose(trials_scheme(bp), stats.norm.isf(1 / np.cumprod(bp)))


def test_next_state_accumulates_complexity_and_survival():
    s0 = initial_state()
    s1 = get_next_state(s0, 2.0, 0.5, 0.9, 4.0)
    assert s1["complexity"] == 4.0 * 0.5 and s1["complexity_cumul"] == 1.0 + 4.0
    np.testing.assert_allclose(s1["success_h1_cumul"], 0.9)
    np.testing.assert_allclose(s1["cost"], 5.0 / 0.9, rtol=1e-6)
    assert s1["threshold_prev"] == -1.0 and not s1["is_empty"]
    s2 = get_next_state(s1, 3.0, 0.25, 0.5, 2.0)
    assert s2["complexity_cumul"] == 5.0 + 2.0 * 2.0
    np.testing.assert_allclose(s2["success_h1_cumul"], 0.45, rtol=1e-6)
    assert s2.dtype == state_dtype


def test_neighbouring_indices_window():
    beam = np.arange(10, 30)
    np.testing.assert_array_equal(neighbouring_indices(beam, 20, 5), [18, 19, 20, 21, 22])
    np.testing.assert_array_equal(neighbouring_indices(beam, 10, 5), [10, 11, 12, 13, 14])
    np.testing.assert_array_equal(neighbouring_indices(beam, 29, 5), [25, 26, 27, 28, 29])
    np.testing.assert_array_equal(neighbouring_indices(beam, 50, 3), [27, 28, 29])


def test_backtrack_best_matches_reference_analyser():
    """backtrack_best against the reference's DynamicThresholdSchemeAnalyser on
    a seeded synthetic design table (tests/golden/schemes_backtrack.npz, made
    by make_fixtures.py --schemes-only)."""
    from conftest import load_golden

    from pyloki_gb300.thresholds import backtrack_best, state_dtype

    d = load_golden("schemes_backtrack")
    states = d["states"].astype(state_dtype)
    paths = backtrack_best(states, d["thresholds"], d["probs"], list(d["min_probs"]))
    assert len(paths) == len(d["min_probs"])
    for i, p in enumerate(paths):
        np.testing.assert_array_equal(p["threshold"], d[f"path_{i}"])
        cost = (p["complexity_cumul"] / p["success_h1_cumul"]).astype(np.float32)
        np.testing.assert_allclose(cost, d[f"cost_{i}"], rtol=1e-6)
    # no final state reaches a survival above 1: empty path, like the reference
    assert len(backtrack_best(states, d["thresholds"], d["probs"], [1.5])[0]) == 0

"""Threshold-scheme design on the GPU: the simulated folds are scored exactly
as the oracle's boxcar S/N scores them, the noise has the requested
statistics, survival rates agree with an independent numpy Monte Carlo of the
reference's procedure, and the dynamic-programming design runs in both modes.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sim(ntrials=2048, seed=1, nbins=64, ducy=0.1, device=None):
    from pyloki_gb300.thresholds import FoldSim, generate_folded_profile

    return FoldSim(generate_folded_profile(nbins=nbins, ducy=ducy), ntrials, 0.2, 1.0,
                   seed=seed, device=device)


@pytest.mark.parametrize("nbins", [64, 50])
def test_scores_equal_oracle_boxcar_of_the_simulated_folds(cuda_device, nbins):
    sim = _sim(nbins=nbins, device=cuda_device)
    (h0, h1), (s0, s1) = sim.run([(None, 0.0), (None, 3.0)], var_add=1.0, var_next=1.0)
    (g0,), (t0,) = sim.run([(h1, 3.0)], var_add=1.0, var_next=2.0)
    for folds, scores, var in ((h0, s0, 1.0), (h1, s1, 1.0), (g0, t0, 2.0)):
        f = folds.cpu().numpy()
        norm = (f / np.sqrt(np.float32(var))).astype(np.float32)
        ref = O.boxcar_snr(norm, sim.widths).max(axis=1)
        np.testing.assert_array_equal(scores, ref)
    # the second generation is the first plus fresh noise and the template
    assert g0.shape[0] == 2048


def test_noise_statistics_and_template(cuda_device):
    from pyloki_gb300.thresholds import generate_folded_profile

    sim = _sim(ntrials=8192, device=cuda_device)
    (h0, h1), _ = sim.run([(None, 0.0), (None, 5.0)], var_add=2.0, var_next=2.0)
    x = h0.cpu().numpy().astype(np.float64)
    n = x.size
    assert abs(x.mean()) < 5 * np.sqrt(2.0 / n)
    assert abs(x.var() - 2.0) < 5 * 2.0 * np.sqrt(2.0 / n)
    # bins are independent: neighbouring-bin correlation is within noise
    c = np.corrcoef(x[:, :-1].ravel(), x[:, 1:].ravel())[0, 1]
    assert abs(c) < 5 / np.sqrt(n)
    prof = generate_folded_profile(nbins=64, ducy=0.1)
    mean1 = h1.cpu().numpy().mean(axis=0)
    np.testing.assert_allclose(mean1, 5.0 * prof, atol=5 * np.sqrt(2.0 / 8192))
    # same seed, same draws; another seed, other draws
    (a,), _ = _sim(ntrials=256, seed=7, device=cuda_device).run([(None, 0.0)], 1.0, 1.0)
    (b,), _ = _sim(ntrials=256, seed=7, device=cuda_device).run([(None, 0.0)], 1.0, 1.0)
    (c2,), _ = _sim(ntrials=256, seed=8, device=cuda_device).run([(None, 0.0)], 1.0, 1.0)
    assert torch.equal(a, b) and not torch.equal(a, c2)


def test_survival_rates_match_numpy_monte_carlo(cuda_device):
    """Two stages of evaluate_scheme against the same procedure with numpy
    normals and the oracle's boxcar (binomial tolerance)."""
    from pyloki_gb300.config import generate_box_width_trials
    from pyloki_gb300.thresholds import evaluate_scheme, generate_folded_profile

    bp, thr, ntrials, snr_final = np.array([2.0, 2.0]), np.array([1.5, 2.5]), 8192, 8.0
    got = evaluate_scheme(thr, bp, 0.1, ntrials=ntrials, snr_final=snr_final, seed=3,
                          device=cuda_device)
    rng = np.random.default_rng(0)
    prof = generate_folded_profile(nbins=64, ducy=0.1)
    widths = generate_box_width_trials(64, ducy_max=0.2, wtsp=1.0)
    bias = snr_final / np.sqrt(len(bp) + 1)
    h = [rng.normal(0, 1, (ntrials, 64)), rng.normal(0, 1, (ntrials, 64)) + bias * prof]
    var = 1.0
    for istage in range(2):
        var += 1.0
        rates = []
        nxt = []
        for k, b in enumerate((0.0, bias)):
            f = np.repeat(h[k], int(np.ceil(ntrials / len(h[k]))), axis=0)[:len(h[k]) * int(
                np.ceil(ntrials / len(h[k])))]
            f = f + rng.normal(0, 1, f.shape) + b * prof
            sc = O.boxcar_snr((f / np.sqrt(var)).astype(np.float32), widths).max(axis=1)
            keep = sc > thr[istage]
            rates.append(keep.mean())
            nxt.append(f[keep])
        h = nxt
        for k, key in enumerate(("success_h0", "success_h1")):
            p = rates[k]
            n = ntrials
            assert abs(got[istage][key] - p) < 6 * np.sqrt(max(p * (1 - p), 1e-4) / n) + 0.01


def test_determine_scheme_keeps_requested_fraction(cuda_device):
    from pyloki_gb300.thresholds import determine_scheme

    probs = np.array([0.5, 0.3, 0.6])
    st = determine_scheme(probs, np.array([2.0, 3.0, 2.0]), 0.1, ntrials=4096, seed=5,
                          device=cuda_device)
    assert len(st) == 3
    np.testing.assert_allclose(st["success_h0"], probs, atol=1e-3)
    assert np.all(np.diff(st["complexity_cumul"]) > 0)
    assert np.all(st["success_h1"] >= st["success_h0"])  # the signal survives more often


@pytest.mark.parametrize("mode", ["improved", "legacy"])
def test_dynamic_scheme_designs_a_path(cuda_device, mode, tmp_path):
    from pyloki_gb300.thresholds import DynamicThresholdScheme

    bp = np.full(6, 2.0)
    ds = DynamicThresholdScheme(bp, 0.1, ntrials=512, nprobs=5, nthresholds=30,
                                snr_final=6.0, beam_width=1.0, mode=mode, seed=2,
                                device=cuda_device)
    ds.run(thres_neigh=5)
    last = ds.states[-1]
    assert (~last["is_empty"]).any()
    ok = ~ds.states["is_empty"]
    s = ds.states[ok]
    np.testing.assert_allclose(s["cost"], s["complexity_cumul"] / s["success_h1_cumul"],
                               rtol=1e-5)
    # each state's H1 survival lies in its probability bin
    for istage in range(ds.nstages):
        for i, k in np.argwhere(~ds.states[istage]["is_empty"]):
            p = ds.states[istage, i, k]["success_h1_cumul"]
            assert ds.probs[k] <= p or np.isclose(ds.probs[k], p)
    path = ds.best_path()
    assert 1 <= len(path) <= ds.nstages
    from pyloki_gb300.thresholds import DynamicThresholdSchemeAnalyser

    saved = ds.save(str(tmp_path))
    assert saved.endswith(".h5")
    an = DynamicThresholdSchemeAnalyser.from_file(saved)
    np.testing.assert_array_equal(an.states, ds.states)
    np.testing.assert_array_equal(an.thresholds, ds.thresholds)
    assert an.beam_width == ds.beam_width
    for a, b in zip(an.backtrack_best([0.1]), ds.backtrack_best([0.1]), strict=True):
        np.testing.assert_array_equal(a, b)


def test_dynamic_scheme_with_unit_first_branching(cuda_device):
    """A pattern that starts with no branching (cumulative trials 1) still
    designs a path: the guess is held at the lowest threshold."""
    from pyloki_gb300.thresholds import DynamicThresholdScheme

    bp = np.array([1.0, 1.0, 3.0, 1.0, 2.0, 3.0])
    ds = DynamicThresholdScheme(bp, 0.1, ntrials=512, nprobs=5, nthresholds=30, snr_final=6.0,
                                beam_width=1.0, mode="improved", seed=4, device=cuda_device)
    ds.run(thres_neigh=5)
    assert (~ds.states[-1]["is_empty"]).any()
    assert 1 <= len(ds.best_path()) <= len(bp)

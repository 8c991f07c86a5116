"""GPU boxcar scoring against the reference fixtures and the oracle (bit-exact)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ["score_nb64", "score_nb50", "score_nb100"]


@pytest.mark.parametrize("name", CASES)
def test_boxcar_snr_matches_reference(cuda_device, name):
    from pyloki_gb300.scoring import boxcar_snr_nd

    d = load_golden(name)
    np.testing.assert_array_equal(boxcar_snr_nd(d["prof"], d["widths"]), d["snr"])
    np.testing.assert_array_equal(boxcar_snr_nd(d["prof"], d["widths"], 1.7), d["snr_std"])


@pytest.mark.parametrize("name", CASES)
def test_snr_score_batch_matches_reference(cuda_device, name):
    from pyloki_gb300.scoring import snr_score_batch

    d = load_golden(name)
    np.testing.assert_array_equal(snr_score_batch(d["comb"], d["widths"]), d["score"])


@pytest.mark.parametrize("nprof", [1, 31, 33, 1000])
@pytest.mark.parametrize("nbins,widths", [(64, [1, 2, 4, 8, 16, 32]), (32, [1, 2, 3, 40]),
                                          (256, [1, 5, 100, 200])])
def test_ragged_counts_and_wide_widths(cuda_device, nprof, nbins, widths):
    """Profile counts off the 32-row tile and widths beyond nbins (extra
    circular wraps of the prefix sum)."""
    import torch

    from pyloki_gb300.scoring import boxcar_snr_nd, snr_score_batch

    rng = np.random.default_rng(nprof + nbins)
    prof = rng.standard_normal((nprof, nbins)).astype(np.float32)
    w = np.array(widths, np.int64)
    np.testing.assert_array_equal(boxcar_snr_nd(prof, w), O.boxcar_snr(prof, w))
    t = torch.from_numpy(prof).to(cuda_device)
    out = boxcar_snr_nd(t, w)
    assert out.is_cuda
    np.testing.assert_array_equal(out.cpu().numpy(), O.boxcar_snr(prof, w))
    comb = np.stack([prof, 1 + rng.random((nprof, nbins)).astype(np.float32)], axis=1)
    np.testing.assert_array_equal(snr_score_batch(comb, w), O.snr_score_batch(comb, w))


def test_empty_bins_nan_semantics(cuda_device):
    """Folds with zero-variance (empty) bins give e / sqrt(0) = NaN or inf
    entries; the NaN propagation and max-skipping must match the reference."""
    from pyloki_gb300.scoring import boxcar_snr_nd, snr_score_batch

    rng = np.random.default_rng(7)
    n, nb = 200, 64
    comb = np.stack([rng.standard_normal((n, nb)), 1 + rng.random((n, nb))], axis=1)
    comb = comb.astype(np.float32)
    comb[::3, 1, ::2] = 0.0          # every other bin empty: 0 / 0 = NaN
    comb[::3, 0, ::2] = 0.0
    comb[1::7, 1, 5] = 0.0           # a single zero variance with e != 0: +-inf
    w = np.array([1, 2, 4, 8, 16, 32], np.int64)
    np.testing.assert_array_equal(snr_score_batch(comb, w), O.snr_score_batch(comb, w))
    norm = O.fold_norm(comb)
    np.testing.assert_array_equal(boxcar_snr_nd(norm, w), O.boxcar_snr(norm, w))


def test_empty_input(cuda_device):
    from pyloki_gb300.scoring import boxcar_snr_nd, snr_score_batch

    out = boxcar_snr_nd(np.zeros((0, 64), np.float32), [1, 2])
    assert out.shape == (0, 2)
    assert snr_score_batch(np.zeros((0, 2, 64), np.float32), [1, 2]).shape == (0,)


def test_nd_shape(cuda_device):
    from pyloki_gb300.scoring import boxcar_snr_nd

    prof = np.random.default_rng(1).standard_normal((3, 4, 5, 64)).astype(np.float32)
    out = boxcar_snr_nd(prof, [1, 2, 4])
    assert out.shape == (3, 4, 5, 3)
    np.testing.assert_array_equal(out, O.boxcar_snr(prof, [1, 2, 4]))

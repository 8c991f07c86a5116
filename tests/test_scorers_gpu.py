"""Alternative scorers and fold variants on the GPU against the reference's
own outputs (``tests/golden/scorers_*.npz``) and the oracle.

Bit-exact: circular Kadane (float64, the reference's order), the bucketed
brute fold. Within stated tolerances: the matched-filter projections (fused
multiply-adds in bin order against numpy's BLAS order), the two-peak and
harmonic scores (float64 here, float32 steps in the reference), and the
oversampled complex fold (cuFFT against numpy's FFT)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import scorer_oracle as O

pytestmark = pytest.mark.gpu

CASES = sorted((Path(__file__).parent / "golden").glob("scorers_*.npz"))
IDS = [p.stem for p in CASES]
PROJ_ATOL = 2e-5      # projections of unit-power templates on |x| < 10 profiles
SCORE_RTOL = 3e-5     # two-peak (same projections) and harmonic scores
DOUBLE_RTOL = 5e-4    # two-peak score against the reference's own projections


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_kadane_bit_exact(cuda_device, path):
    from pyloki_gb300.scoring import kadane_circular_normalized

    z = np.load(path)
    snr, w, s = kadane_circular_normalized(z["profiles"], z["biases"], device=cuda_device)
    np.testing.assert_array_equal(snr, z["kadane_snr"])
    np.testing.assert_array_equal(w, z["kadane_width"])
    np.testing.assert_array_equal(s, z["kadane_start"])


def test_kadane_random_against_oracle(cuda_device):
    from pyloki_gb300.scoring import kadane_circular_normalized

    rng = np.random.default_rng(4)
    prof = rng.standard_normal((300, 100)).astype(np.float32)
    prof[::7, 95:] += 3.0  # wrapped windows
    prof[::7, :4] += 3.0
    biases = np.array([0.0, 0.1, 0.3], np.float32)
    snr, w, s = kadane_circular_normalized(prof, biases, device=cuda_device)
    ref = [O.kadane(x, biases) for x in prof]
    np.testing.assert_array_equal(snr, [r[0] for r in ref])
    np.testing.assert_array_equal(w, [r[1] for r in ref])
    np.testing.assert_array_equal(s, [r[2] for r in ref])
    assert (w[::7] > 4).all()


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_matched_filter_bank(cuda_device, path):
    from pyloki_gb300.scoring import MatchedFilter

    z = np.load(path)
    nb = int(z["nbins"])
    prof = z["profiles"]
    for kind in ("boxcar", "gaussian"):
        mf = MatchedFilter(z["mf_widths"], nb, 1, kind)
        # the reference normalises templates with numpy's mean and BLAS dot,
        # whose summation order is the machine's: a few ulps between hosts
        np.testing.assert_allclose(mf.e_mat, z[f"{kind}_e_mat"], rtol=0, atol=2e-6)
        mf.e_mat = z[f"{kind}_e_mat"]  # score with the reference's exact bank
        np.testing.assert_allclose(mf.compute_snr(prof, device=cuda_device), z[f"{kind}_snr"],
                                   rtol=0, atol=PROJ_ATOL)
        np.testing.assert_allclose(mf.compute_dot(prof.T, device=cuda_device),
                                   z[f"{kind}_dot"], rtol=0, atol=PROJ_ATOL)
        mf.templates = z[f"{kind}_templates"]
        np.testing.assert_allclose(mf.compute_fft(prof, device=cuda_device), z[f"{kind}_fft"],
                                   rtol=0, atol=PROJ_ATOL)
        dbl = mf.compute_dot_double(prof, device=cuda_device)
        # from the GPU's own projections the oracle gives the same score
        proj = mf.compute_dot(prof.T, device=cuda_device).T
        ref = O.snr_double_from_scores(proj, np.dot(mf.e_mat, mf.e_mat.T))
        np.testing.assert_allclose(dbl, ref, rtol=SCORE_RTOL)
        # against the reference: the pair score divides by 1 - gamma^2 and
        # cancels for nearly collinear filters, so the projections' last-ulp
        # differences (bin-order FMA here, BLAS there) grow ~100-fold
        np.testing.assert_allclose(dbl, z[f"{kind}_double"], rtol=DOUBLE_RTOL)
    mf = MatchedFilter(np.array([2, 6]), nb, int(z["shift"]), "boxcar")
    mf.e_mat = z["shift_e_mat"]
    np.testing.assert_allclose(mf.compute_snr(prof, device=cuda_device), z["shift_snr"], rtol=0,
                               atol=PROJ_ATOL)
    # one profile, device tensors in and out
    t = torch.from_numpy(prof[:3]).to(cuda_device)
    out = mf.compute_snr(t)
    assert isinstance(out, torch.Tensor) and out.shape == (3, 2)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_harmonic_summing(cuda_device, path):
    from pyloki_gb300.scoring import harmonic_summing_score

    z = np.load(path)
    got = np.stack([harmonic_summing_score(z["harm_folds"], int(nh), device=cuda_device)
                    for nh in z["harm_nh"]], axis=1)
    np.testing.assert_allclose(got, z["harmonic"], rtol=SCORE_RTOL)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_bucketed_and_oversampled_folds(cuda_device, path):
    from pyloki_gb300.ffa import brutefold_bucketed, brutefold_complex_oversampled

    z = np.load(path)
    nb = int(z["nbins"])
    args = [torch.from_numpy(z[k]).to(cuda_device) for k in ("bf_ts_e", "bf_ts_v", "bf_freqs")]
    kw = dict(segment_len=int(z["bf_segment_len"]), nbins=nb, tsamp=float(z["bf_tsamp"]),
              t_ref=float(z["bf_t_ref"]))
    np.testing.assert_array_equal(brutefold_bucketed(*args, **kw).cpu().numpy(), z["bucketed"])
    got = brutefold_complex_oversampled(*args, **kw).cpu().numpy()
    ref = z["oversampled"]
    assert got.shape == ref.shape and got.dtype == np.complex64
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-5 * np.abs(ref).max())
    with pytest.raises(ValueError, match="multiple of the segment length"):
        brutefold_bucketed(args[0][:-1], args[1][:-1], args[2], **kw)


def test_empty_inputs(cuda_device):
    from pyloki_gb300.scoring import MatchedFilter, kadane_circular_normalized

    e = np.zeros((0, 64), np.float32)
    snr, w, s = kadane_circular_normalized(e, np.zeros(1, np.float32), device=cuda_device)
    assert snr.shape == (0,)
    assert MatchedFilter([1, 2], 64).compute_snr(e, device=cuda_device).shape == (0, 2)

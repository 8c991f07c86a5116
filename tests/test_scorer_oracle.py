"""The alternative-scorer oracle against the reference's own outputs
(``tests/golden/scorers_*.npz``): circular Kadane bit for bit; the matched-
filter bank, the two-peak score and harmonic summing to float32-level
tolerances (the reference computes those in float32 where this oracle, like
the GPU, carries float64)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import scorer_oracle as O

CASES = sorted((Path(__file__).parent / "golden").glob("scorers_*.npz"))


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_scorer_oracle_against_reference(path):
    z = np.load(path)
    prof = z["profiles"]
    res = [O.kadane(x, z["biases"]) for x in prof]
    np.testing.assert_array_equal([r[0] for r in res], z["kadane_snr"])
    np.testing.assert_array_equal([r[1] for r in res], z["kadane_width"])
    np.testing.assert_array_equal([r[2] for r in res], z["kadane_start"])
    for kind in ("boxcar", "gaussian"):
        e = z[f"{kind}_e_mat"]
        np.testing.assert_allclose(O.snr_e_mat_2d(prof, e, np.ones(7, np.int64)),
                                   z[f"{kind}_snr"], rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(O.snr_double(prof, e), z[f"{kind}_double"], rtol=2e-5)
        np.testing.assert_allclose(O.snr_fft(prof, z[f"{kind}_templates"]), z[f"{kind}_fft"],
                                   rtol=0, atol=1e-5)
    sh = np.full(2, int(z["shift"]), np.int64)
    np.testing.assert_allclose(O.snr_e_mat_2d(prof, z["shift_e_mat"], sh), z["shift_snr"],
                               rtol=1e-6, atol=1e-6)
    got = np.array([[O.harmonic(f, nh) for nh in z["harm_nh"]] for f in z["harm_folds"]])
    np.testing.assert_allclose(got, z["harmonic"], rtol=2e-5)


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_template_banks_equal_reference(path):
    """Host-built banks against the reference's on this host (numpy's mean
    and BLAS dot set the last ulps, so another host may differ by a few)."""
    from pyloki_gb300.scoring import MatchedFilter

    z = np.load(path)
    nb = int(z["nbins"])
    for kind in ("boxcar", "gaussian"):
        mf = MatchedFilter(z["mf_widths"], nb, 1, kind)
        np.testing.assert_array_equal(mf.templates, z[f"{kind}_templates"])
        np.testing.assert_array_equal(mf.e_mat, z[f"{kind}_e_mat"])
    mf = MatchedFilter(np.array([2, 6]), nb, int(z["shift"]), "boxcar")
    np.testing.assert_array_equal(mf.e_mat, z["shift_e_mat"])

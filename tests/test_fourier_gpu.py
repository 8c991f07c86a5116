"""Fourier-domain FFA (use_fourier=True) against the pyloki reference.

The reference folds through a float32 BLAS product, numpy's float32 cos/sin
and pocketfft's inverse transform; the GPU evaluates the same float32
expressions with its own summation order and CUDA's sincos, so this path is
compared to a float32 tolerance: every complex fold row, normalised profile
and S/N row must agree with the reference to TOL of that row's largest
magnitude.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ["ffa_freq_fourier", "ffa_accel_fourier"]
TOL_FOLD = 2e-5
TOL_NORM = 2e-5
TOL_SNR = 2e-5


def _rel_err(got, ref):
    """Largest |got - ref| of every row over the row's largest |ref|."""
    g = np.asarray(got).reshape(-1, np.asarray(got).shape[-1])
    r = np.asarray(ref).reshape(-1, np.asarray(ref).shape[-1])
    scale = np.abs(r).max(axis=1)
    scale[scale == 0] = 1.0
    return float((np.abs(g - r).max(axis=1) / scale).max())


@pytest.mark.parametrize("name", CASES)
def test_fourier_levels_norm_and_snr(cuda_device, name):
    from pyloki_gb300.config import PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.scoring import boxcar_snr_nd
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=True)
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device)
    dyp.initialize()
    errs = {0: _rel_err(dyp.fold.cpu().numpy(), d["fold_0"])}
    for lvl in range(1, int(d["niters"]) + 1):
        dyp._execute_iter()
        errs[lvl] = _rel_err(dyp.fold.cpu().numpy(), d[f"fold_{lvl}"])
    norm = dyp.get_fold_norm()
    e_norm = _rel_err(norm.cpu().numpy(), d["fold_norm"])
    snr = boxcar_snr_nd(norm, d["widths"], 1.0)
    e_snr = _rel_err(snr.cpu().numpy(), d["snrs"])
    print(name, "fold", errs, "norm", e_norm, "snr", e_snr)
    assert max(errs.values()) <= TOL_FOLD, errs
    assert e_norm <= TOL_NORM
    assert e_snr <= TOL_SNR
    # the best trial is the reference's best trial
    assert np.argmax(snr.cpu().numpy()) == np.argmax(d["snrs"])


def test_fourier_search_matches_materialised(cuda_device):
    """search() on the Fourier path = levels + irfft norm + boxcar."""
    from pyloki_gb300.config import PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden("ffa_accel_fourier")
    cfg = PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=True)
    ts = TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp)
    snr = DynamicProgramming(ts, cfg, device=cuda_device).search()
    assert _rel_err(snr.cpu().numpy(), d["snrs"]) <= TOL_SNR

"""TimeSeries.fold_ephem and downsample on the GPU against the reference's
own outputs (``tests/golden/timeseries_ephem.npz``): the folds bit for bit
(every (subint, bin) summed in sample order), the normalised profiles bit
for bit, the downsampled series to float32 rounding (the reference's numpy
mean sums pairwise in float32, the kernel in float64)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

Z = Path(__file__).parent / "golden" / "timeseries_ephem.npz"


def _ts(z, device=None):
    from pyloki_gb300.timeseries import TimeSeries

    e, v = z["ts_e"], z["ts_v"]
    if device is not None:
        e, v = torch.from_numpy(e).to(device), torch.from_numpy(v).to(device)
    return TimeSeries(e, v, float(z["dt"]))


def test_fold_ephem_bit_exact(cuda_device):
    z = np.load(Z)
    ts = _ts(z)
    f0 = float(z["freq"])
    kw = {"mod_kwargs": {"acc": 12.0, "jerk": 0.3}, "device": cuda_device}
    np.testing.assert_array_equal(ts.fold_ephem(f0, 64, 1, normalize=False, **kw), z["fold1"])
    np.testing.assert_array_equal(ts.fold_ephem(f0, 64, 1, **kw), z["norm1"])
    np.testing.assert_array_equal(ts.fold_ephem(f0, 50, 8, normalize=False, **kw), z["fold8"])
    np.testing.assert_array_equal(ts.fold_ephem(f0, 50, 8, **kw), z["norm8"])
    circ = ts.fold_ephem(f0, 32, 3, normalize=False, mod_type="circular",
                         mod_kwargs={"p_orb": 600.0, "x_orb": 0.01, "psi": 0.2},
                         device=cuda_device)
    np.testing.assert_array_equal(circ, z["fold_circ"])
    # device tensors in, device tensors out
    out = _ts(z, cuda_device).fold_ephem(f0, 64, 1, **kw)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    np.testing.assert_array_equal(out.cpu().numpy(), z["norm1"])


def test_downsample(cuda_device):
    z = np.load(Z)
    ds = _ts(z).downsample(4, device=cuda_device)
    np.testing.assert_allclose(ds.ts_e, z["ds_e"], rtol=2e-6, atol=2e-7)
    np.testing.assert_allclose(ds.ts_v, z["ds_v"], rtol=2e-6, atol=2e-7)
    assert ds.dt == float(z["ds_dt"])  # the reference keeps the sampling time


def test_fold_ephem_argument_checks(cuda_device):
    z = np.load(Z)
    ts = _ts(z)
    with pytest.raises(ValueError, match="less than the total"):
        ts.fold_ephem(0.01, 64, device=cuda_device)
    with pytest.raises(ValueError, match="subints must be"):
        ts.fold_ephem(float(z["freq"]), 64, 10**6, device=cuda_device)

"""Series conditioning on the GPU (TimeSeries.deredden / normalise / from_tim,
io/timeseries.py:198-236) against CPU restatements of the definitions the
library documents: scipy.ndimage.median_filter (mode "reflect") for the
running median, numpy's partition / percentile / mean / std for the order
statistics and scales. Running medians and order statistics are exact
(bit-identical); the float64 mean and the scales to 1e-12 relative; the
normalised series to 2 float32 ulps. Parity with the reference's own
from_tim is unpinned: its filters live in sigpyproc, which is absent."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _median_filter(x, w):
    from scipy import ndimage

    return ndimage.median_filter(x, size=w, mode="reflect")


@pytest.mark.parametrize("n,w", [(1, 1), (7, 4), (5, 9), (1000, 1), (1000, 2), (1000, 3),
                                 (3001, 64), (20000, 501), (20000, 2048), (9000, 4999),
                                 (40000, 16384)])
def test_running_median_matches_definition(cuda_device, n, w):
    from pyloki_gb300 import _lib

    rng = np.random.default_rng(n + w)
    x = rng.standard_normal(n).astype(np.float32)
    if n > 100:
        x[::7] = np.round(x[::7])  # ties
    xd = torch.from_numpy(x).to(cuda_device)
    out = torch.empty_like(xd)
    lib = _lib.load()
    stream = _lib.stream_ptr(torch.cuda.current_stream(cuda_device))
    want = _median_filter(x, w)
    _lib.check(lib.loki_running_median(_lib.ptr(xd), n, w, 0, _lib.ptr(out), stream))
    np.testing.assert_array_equal(out.cpu().numpy(), want)
    _lib.check(lib.loki_running_median(_lib.ptr(xd), n, w, 1, _lib.ptr(out), stream))
    np.testing.assert_array_equal(out.cpu().numpy(), x - want)


def test_running_median_rejects_bad_windows(cuda_device):
    from pyloki_gb300 import _lib

    lib = _lib.load()
    xd = torch.zeros(10, device=cuda_device)
    with pytest.raises(ValueError, match="must be >= 1"):
        _lib.check(lib.loki_running_median(_lib.ptr(xd), 10, 0, 0, _lib.ptr(xd), 0))
    with pytest.raises(NotImplementedError, match="above 32768"):
        _lib.check(lib.loki_running_median(_lib.ptr(xd), 10, 32769, 0, _lib.ptr(xd), 0))


@pytest.mark.parametrize("n", [1, 2, 5, 1000, 2**20 + 3])
def test_select_kth_matches_partition(cuda_device, n):
    from pyloki_gb300.timeseries import _Stats

    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) * 10).astype(np.float32)
    if n > 10:
        x[: n // 3] = np.round(x[: n // 3])
        x[5] = np.inf
        x[6] = -np.inf
    st = _Stats(torch.from_numpy(x).to(cuda_device), cuda_device)
    s = np.sort(x)
    for k in sorted({0, n // 4, n // 2, n - 1, max(0, n - 2)}):
        assert st.kth(k) == s[k], k


def test_statistics_match_numpy(cuda_device):
    from pyloki_gb300.timeseries import _Stats

    rng = np.random.default_rng(5)
    x = (rng.standard_normal(100003) * 3 + 1).astype(np.float32)
    st = _Stats(torch.from_numpy(x).to(cuda_device), cuda_device)
    xd = x.astype(np.float64)
    assert abs(st.mean() - xd.mean()) <= 1e-12 * abs(xd.mean())
    assert abs(st.std() - (x - np.float32(xd.mean())).astype(np.float64).std()) <= 1e-12
    assert st.median() == np.median(x)
    for q in (25.0, 75.0, 10.0):
        assert abs(st.percentile(q) - float(np.percentile(xd, q))) <= 1e-6 * abs(
            np.percentile(xd, q)) + 1e-7
    mad = np.median(np.abs(x - np.float32(np.median(x))))
    assert st.mad() == mad


@pytest.mark.parametrize("scale", ["iqr", "std", "mad"])
@pytest.mark.parametrize("tim_type", ["dat", "tim"])
def test_from_tim_matches_restatement(cuda_device, tmp_path, scale, tim_type):
    """A seeded series with red noise and a pulsar, written as .dat or .tim,
    loaded by from_tim: the deredden and normalisation steps against the
    numpy / scipy restatement."""
    from pyloki_gb300 import sigproc
    from pyloki_gb300.timeseries import TimeSeries

    rng = np.random.default_rng(11)
    n, tsamp = 2**16, 5e-4
    t = np.arange(n) * tsamp
    red = np.cumsum(rng.standard_normal(n)) * 0.05
    x = (rng.standard_normal(n) + red + 0.5 * (np.sin(2 * np.pi * 7.3 * t) > 0.95)).astype(
        np.float32)
    path = tmp_path / f"s.{tim_type}"
    (sigproc.write_dat if tim_type == "dat" else sigproc.write_tim)(path, x, tsamp)
    ts = TimeSeries.from_tim(path, tim_type=tim_type, filter_window=0.5,
                             norm_scale_method=scale)
    w = int(0.5 / tsamp)
    d = x - _median_filter(x, w)
    loc = np.float32(d.astype(np.float64).mean())
    if scale == "iqr":
        s = (np.percentile(d.astype(np.float64), 75) - np.percentile(d.astype(np.float64), 25)
             ) / 1.3489795003921634
    elif scale == "std":
        s = (d - loc).astype(np.float64).std()
    else:
        s = np.median(np.abs(d - np.float32(np.median(d)))) * 1.482602218505602
    want = (d - loc) / np.float32(s)
    np.testing.assert_allclose(ts.ts_e, want, rtol=0, atol=2 * np.spacing(np.abs(want).max()))
    np.testing.assert_array_equal(ts.ts_v, np.ones(n, np.float32))
    assert ts.tsamp == tsamp and ts.nsamps == n

"""The unit-variance brute fold (ts_v all ones: variance sums from sample
counts) equals the general fold bit for bit: full and partial last
segments, chunked phase scratch, 8-bit and 16-bit phase maps; and
DynamicProgramming takes it exactly when ts_v is all ones."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nsamps,seg,nbins,scratch", [
    (2**16, 4096, 64, 1 << 30),         # whole segments
    (2**16 + 1234, 4096, 64, 1 << 30),  # a shorter last segment
    (2**15, 2048, 64, 3 * 2048),        # three frequencies per scratch chunk
    (2**15 + 77, 2048, 300, 1 << 30),   # 16-bit phase map
])
def test_unit_variance_fold_equals_general(cuda_device, nsamps, seg, nbins, scratch):
    from pyloki_gb300.ffa import brutefold

    rng = np.random.default_rng(nsamps + nbins)
    e = torch.from_numpy(rng.standard_normal(nsamps).astype(np.float32)).to(cuda_device)
    v = torch.ones(nsamps, dtype=torch.float32, device=cuda_device)
    freqs = torch.from_numpy(np.linspace(3.0, 41.0, 37)).to(cuda_device)
    kw = dict(segment_len=seg, nbins=nbins, tsamp=1e-3, t_ref=0.7, scratch_bytes=scratch)
    a = brutefold(e, v, freqs, **kw)
    b = brutefold(e, v, freqs, unit_variance=True, **kw)
    assert torch.equal(a, b)


def test_dynamic_programming_detects_unit_variance(cuda_device):
    from pyloki_gb300 import PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    n = 2**15
    cfg = PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
                             param_limits=[(10.0, 14.0)], ducy_max=0.5, wtsp=2.0,
                             use_fourier=False)
    rng = np.random.default_rng(3)
    e = rng.standard_normal(n).astype(np.float32)
    ones = DynamicProgramming(TimeSeries(e, np.ones(n, np.float32), cfg.tsamp), cfg,
                              device=cuda_device)
    ones.initialize()
    general = DynamicProgramming(TimeSeries(e, np.ones(n, np.float32), cfg.tsamp), cfg,
                                 device=cuda_device, unit_variance=False)
    general.initialize()
    assert ones._unit_var and not general._unit_var
    assert torch.equal(ones.fold, general.fold)
    v = np.ones(n, np.float32)
    v[17] = 1.5
    other = DynamicProgramming(TimeSeries(e, v, cfg.tsamp), cfg, device=cuda_device)
    other.initialize()
    assert not other._unit_var
    dev_v = DynamicProgramming(TimeSeries(torch.from_numpy(e).to(cuda_device),
                                          torch.ones(n, device=cuda_device), cfg.tsamp), cfg,
                               device=cuda_device)
    dev_v.initialize()
    assert dev_v._unit_var


def test_complex_fold_unit_variance_equals_general(cuda_device):
    """ts_v NULL (all ones) gives the same complex fold as ts_v = ones."""
    from pyloki_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(9)
    n, seg, nbins = 2**14 * 5, 2**14, 64
    e = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).to(cuda_device)
    v = torch.ones(n, dtype=torch.float32, device=cuda_device)
    freqs = torch.from_numpy(np.linspace(5.0, 60.0, 23)).to(cuda_device)
    out = [torch.empty((n // seg, 23, 2, nbins // 2 + 1), dtype=torch.complex64,
                       device=cuda_device) for _ in range(2)]
    stream = _lib.stream_ptr(torch.cuda.current_stream(cuda_device))
    for vp, o in ((v, out[0]), (None, out[1])):
        _lib.check(lib.loki_brutefold_complex(_lib.ptr(e), _lib.ptr(vp), n, _lib.ptr(freqs), 23,
                                              seg, nbins, 1e-3, 0.5 * seg * 1e-3, _lib.ptr(o),
                                              stream))
    assert torch.equal(out[0], out[1])

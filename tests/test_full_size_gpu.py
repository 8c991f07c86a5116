"""Full-size parity: the benchmark searches themselves, checked bit for bit on
sampled trials against the oracle's single-trial recursion (one pass over the
series per trial, so any trial of a full-size search can be re-derived).

- the 2^23-sample acceleration search of the benchmark (1.49e9 trials,
  banded final levels);
- a 2^21-sample jerk search of the batch workload's grids, alone and stacked
  with a second series (``nbatch=2``).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _check(snr, ts_e, ts_v, cfg, n_random=96, seed=0):
    flat = snr.reshape(-1, snr.shape[-1])
    best = torch.nan_to_num(flat.amax(dim=1), nan=float("-inf"))
    top = torch.topk(best, 8).indices.cpu().numpy()
    rng = np.random.default_rng(seed)
    pick = np.unique(np.r_[top, rng.integers(0, flat.shape[0], n_random)])
    got = flat[torch.from_numpy(pick).to(flat.device)].cpu().numpy()
    ref = O.boxcar_snr(O.fold_norm(O.ffa_trials(ts_e, ts_v, cfg, pick)), cfg.score_widths)
    np.testing.assert_array_equal(got, ref)


def test_benchmark_accel_search_2e23_spot_trials_bit_exact(cuda_device):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.simulation import make_series

    n = 2**23
    cfg = PulsarSearchConfig(
        nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
        param_limits=ParamLimits.from_taylor((50.0, 500.0), accel=(-50.0, 50.0)).limits,
        ducy_max=0.25, wtsp=2.0, use_fourier=False, bseg_brute=16384)
    ts = make_series(n, 64e-6, freq=200.0, snr=15.0, ducy=0.05, accel=20.0, seed=1000)
    dyp = DynamicProgramming(ts, cfg, device=cuda_device)
    snr = dyp.search()
    assert tuple(snr.shape) == (193, 7730942, 5)
    _check(snr, ts.ts_e, ts.ts_v, cfg)
    # the fast normalisation: every trial within 1e-5 of the exact search
    # (relative to max(|S/N|, 1)), the same NaN pattern (empty-bin trials)
    fast = DynamicProgramming(ts, cfg, device=cuda_device).search(norm="fast")
    a, b = snr.reshape(-1), fast.reshape(-1)
    err = 0.0
    for i in range(0, a.numel(), 1 << 28):  # chunks of 1 GiB
        x, y = a[i:i + (1 << 28)], b[i:i + (1 << 28)]
        fin = torch.isfinite(x)
        assert torch.equal(fin, torch.isfinite(y))
        d = torch.where(fin, (y - x).abs() / x.abs().clamp(min=1.0), torch.zeros_like(x))
        err = max(err, d.max().item())
    assert err <= 1e-5, err


def test_jerk_search_2e21_spot_trials_bit_exact_single_and_stacked(cuda_device):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.simulation import make_series
    from pyloki_gb300.timeseries import TimeSeries

    n = 2**21
    cfg = PulsarSearchConfig(
        nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
        param_limits=ParamLimits.from_taylor((50.0, 500.0), accel=(-30.0, 30.0),
                                             jerk=(-0.05, 0.05)).limits,
        ducy_max=0.25, wtsp=2.0, use_fourier=False, bseg_brute=16384)
    a = make_series(n, 64e-6, freq=300.0, snr=12.0, ducy=0.05, accel=10.0, jerk=0.02, seed=7)
    b = make_series(n, 64e-6, seed=8)
    one = DynamicProgramming(a, cfg, device=cuda_device).search()
    _check(one, a.ts_e, a.ts_v, cfg, seed=1)
    both = DynamicProgramming(TimeSeries(np.concatenate([a.ts_e, b.ts_e]),
                                         np.concatenate([a.ts_v, b.ts_v]), cfg.tsamp),
                              cfg, device=cuda_device, nbatch=2).search()
    # equal arrays, NaN (empty-bin trials) included
    np.testing.assert_array_equal(both[0].cpu().numpy(), one.cpu().numpy())
    _check(both[1], b.ts_e, b.ts_v, cfg, seed=2)

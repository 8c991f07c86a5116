"""The vectorised Taylor level descriptors equal the per-level ones byte for
byte (host only: a stand-in holds the attributes the builders read)."""

from __future__ import annotations

import ctypes as C
import types

import numpy as np
import pytest


@pytest.mark.parametrize("moving", [True, False])
@pytest.mark.parametrize("tiling", ["aggressive", "quadrature", "conservative"])
def test_vectorised_descriptors_equal_per_level(moving, tiling):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.prune import Pruning
    from pyloki_gb300.scheme import MiddleOutScheme

    n = 2**18
    limits = ParamLimits.from_taylor((150.0, 151.0), accel=(-5.0, 5.0), jerk=(-1e-3, 1e-3),
                                     snap=(-1e-7, 1e-7)).limits
    cfg = PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0, param_limits=limits,
                             ducy_max=0.25, wtsp=1.5, use_fourier=False, bseg_brute=2048,
                             bseg_ffa=n // 32, tiling_strategy=tiling)
    nseg = 32
    fake = types.SimpleNamespace(
        dyp=types.SimpleNamespace(cfg=cfg, nsegments=nseg),
        scheme=MiddleOutScheme(nseg, 11, cfg.bseg_ffa * cfg.tsamp, 1),
        use_moving_grid=moving, poly_order=4, nparams_ffa=4,
        param_grid_count_init=np.array([3, 5, 7, 11]), poly_basis="taylor", circular=False)
    arr = Pruning._level_descs_taylor(fake, nseg - 1)
    for level in range(1, nseg):
        one = Pruning._level_desc(fake, level)
        assert bytes(arr[level - 1]) == bytes(one), level
        assert C.sizeof(one) == C.sizeof(arr[level - 1])


@pytest.mark.parametrize("moving", [True, False])
def test_vectorised_descriptors_circular(moving):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.prune import Pruning
    from pyloki_gb300.scheme import MiddleOutScheme

    n = 2**18
    pl = ParamLimits.from_circular((333.0, 334.0), 7200.0, poly_order=5)
    cfg = PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
                             param_limits=pl.limits, ducy_max=0.25, wtsp=1.5,
                             use_fourier=False, bseg_brute=2048, bseg_ffa=n // 16,
                             p_orb_min=7200.0)
    nseg = 16
    fake = types.SimpleNamespace(
        dyp=types.SimpleNamespace(cfg=cfg, nsegments=nseg),
        scheme=MiddleOutScheme(nseg, 5, cfg.bseg_ffa * cfg.tsamp, 1),
        use_moving_grid=moving, poly_order=5, nparams_ffa=5,
        param_grid_count_init=np.array([2, 3, 5, 7, 11]), poly_basis="taylor", circular=True)
    arr = Pruning._level_descs_taylor(fake, nseg - 1)
    for level in range(1, nseg):
        assert bytes(arr[level - 1]) == bytes(Pruning._level_desc(fake, level)), level

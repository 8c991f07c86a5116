"""Host-side grid arithmetic against the reference's grids."""

from __future__ import annotations

import numpy as np
import pytest

from pyloki_gb300.config import ParamLimits, PulsarSearchConfig, generate_box_width_trials
from tests.conftest import cfg_from_golden, load_golden


@pytest.mark.parametrize("name", ["ffa_freq", "ffa_accel", "ffa_jerk"])
def test_grids_match_reference(name):
    d = load_golden(name)
    cfg = cfg_from_golden(d)
    assert cfg.bseg_brute == int(d["bseg_brute"])
    assert cfg.bseg_ffa == int(d["bseg_ffa"])
    assert cfg.niters_ffa == int(d["niters"])
    np.testing.assert_array_equal(cfg.score_widths, d["widths"])
    for lvl in range(cfg.niters_ffa + 1):
        np.testing.assert_array_equal(cfg.get_param_grid_count(lvl), d[f"counts_{lvl}"])
        np.testing.assert_array_equal(cfg.get_dparams(lvl), d[f"dparams_{lvl}"])
        for ip, arr in enumerate(cfg.get_param_arr(cfg.get_dparams(lvl))):
            np.testing.assert_array_equal(arr, d[f"param_{lvl}_{ip}"])


@pytest.mark.parametrize("name", ["score_nb64", "score_nb50", "score_nb100"])
def test_width_trials(name):
    d = load_golden(name)
    nb = {"score_nb64": (64, 0.5, 2.0), "score_nb50": (50, 0.2, 1.5),
          "score_nb100": (100, 0.3, 1.3)}[name]
    np.testing.assert_array_equal(generate_box_width_trials(*nb), d["widths"])


def test_accel_search_sizes():
    """The 2^23-sample acceleration search: 9 levels, 193 x 7730942 final trials."""
    cfg = PulsarSearchConfig(nsamps=2**23, tsamp=64e-6, nbins=64, eta=1.0,
                             param_limits=ParamLimits.from_taylor((50.0, 500.0),
                                                                  accel=(-50.0, 50.0)).limits,
                             ducy_max=0.25, wtsp=2.0, use_fourier=False)
    assert cfg.bseg_brute == 16384
    assert cfg.niters_ffa == 9
    np.testing.assert_array_equal(cfg.get_param_grid_count(9), [193, 7730942])
    np.testing.assert_array_equal(cfg.score_widths, [1, 2, 4, 8, 16])


def test_validation_errors():
    lim = [(1.0, 10.0)]
    with pytest.raises(ValueError):
        PulsarSearchConfig(nsamps=1000, tsamp=1e-3, nbins=64, eta=1.0, param_limits=lim)
    with pytest.raises(ValueError):
        PulsarSearchConfig(nsamps=2**16, tsamp=1e-3, nbins=64, eta=1.0,
                           param_limits=[(10.0, 1.0)])
    with pytest.raises(ValueError):
        PulsarSearchConfig(nsamps=2**16, tsamp=1e-3, nbins=64, eta=1.0, param_limits=lim,
                           bseg_brute=2**10, bseg_ffa=2**9)
    with pytest.raises(ValueError):
        PulsarSearchConfig(nsamps=2**16, tsamp=1e-3, nbins=64, eta=1.0, param_limits=lim,
                           tiling_strategy="bogus")
    with pytest.raises(ValueError):
        PulsarSearchConfig(nsamps=2**16, tsamp=1e-3, nbins=64, eta=1.0,
                           param_limits=[(0.0, 1.0), (1.0, 10.0)], prune_poly_order=5)


def test_limit_factories():
    lim = ParamLimits.from_taylor((1.0, 2.0), accel=(-3.0, 3.0))
    np.testing.assert_array_equal(lim.limits, [[-3.0, 3.0], [1.0, 2.0]])
    lim = ParamLimits.from_taylor((1.0, 2.0), jerk=(-1.0, 1.0))
    np.testing.assert_array_equal(lim.limits, [[-1.0, 1.0], [0.0, 0.0], [1.0, 2.0]])
    circ = ParamLimits.from_circular(333.33, p_orb_min=7200.0, poly_order=4)
    assert circ.limits.shape == (4, 2)
    assert circ.limits[-1, 0] < 333.33 < circ.limits[-1, 1]

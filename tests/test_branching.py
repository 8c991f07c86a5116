"""Branching pattern of the Taylor tree against the reference.

``tests/golden/branching_taylor4.npz`` holds the reference's
``generate_branching_pattern`` for the circular-orbit benchmark search
(Taylor tree to the 4th derivative, 2^22 samples, 128 segments), made by
``make_fixtures.py --branching-only``. The host restatement must match it
bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden

CASES = [("moving_64", "aggressive", "poly_taylor_moving", 64),
         ("moving_0", "aggressive", "poly_taylor_moving", 0),
         ("moving_100", "aggressive", "poly_taylor_moving", 100),
         ("fixed_64", "aggressive", "poly_taylor_fixed", 64),
         ("quad_64", "quadrature", "poly_taylor_moving", 64),
         ("cons_64", "conservative", "poly_taylor_moving", 64)]


@pytest.mark.parametrize(("key", "tiling", "kind", "ref"), CASES)
def test_branching_pattern_matches_reference(key, tiling, kind, ref):
    from pyloki_gb300 import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.branching import generate_branching_pattern

    d = load_golden("branching_taylor4")
    n = 2**22
    lim = ParamLimits.from_circular(333.33, p_orb_min=7200.0, poly_order=4)
    np.testing.assert_array_equal(lim.limits, d["param_limits"])
    cfg = PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0, param_limits=lim.limits,
                             use_fourier=False, bseg_ffa=n // 128, prune_poly_order=4,
                             tiling_strategy=tiling)
    got = generate_branching_pattern(cfg, kind, ref_seg=ref)
    np.testing.assert_array_equal(got, d[key])


def test_branching_pattern_rejects_unknown_kind():
    import bench
    from pyloki_gb300.branching import generate_branching_pattern

    with pytest.raises(ValueError, match="Invalid kind"):
        generate_branching_pattern(bench.make_prune_cfg(), "poly_spline_moving")

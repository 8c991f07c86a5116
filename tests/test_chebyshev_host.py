"""Chebyshev-basis host math against the reference runs (no GPU).

The seed leaves and the final report are computed on the host with numpy, as
the reference does; the per-level matrices feed the GPU kernels.
"""

from __future__ import annotations

import numpy as np
import pytest

from pyloki_gb300 import chebyshev
from tests.conftest import load_golden

CASES = ["prune_cheby", "prune_cheby_fixed", "prune_cheby_cons", "prune_cheby_quad"]
TILING = {"prune_cheby_cons": "conservative", "prune_cheby_quad": "quadrature"}


def _cfg(d, name):
    from pyloki_gb300.config import PulsarSearchConfig

    return PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=False, bseg_ffa=int(d["bseg_ffa"]),
        prune_poly_order=int(d["poly_order"]), branch_max=int(d["branch_max"]),
        tiling_strategy=TILING.get(name, "aggressive"))


@pytest.mark.parametrize("name", CASES)
def test_seed_leaves_match_reference(name):
    from pyloki_gb300.scheme import MiddleOutScheme

    d = load_golden(name)
    cfg = _cfg(d, name)
    n = cfg.niters_ffa
    nseg = cfg.nsamps // cfg.bseg_ffa
    sc = MiddleOutScheme(nseg, int(d["ref_seg"]), cfg.tseg_ffa, 1)
    leaves = chebyshev.seed_leaves(cfg.get_param_arr(cfg.get_dparams(n)),
                                   cfg.get_dparams_actual(n), cfg.prune_poly_order,
                                   sc.get_coord(0)[1])
    np.testing.assert_allclose(leaves, d["seed_leaves"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", CASES)
def test_report_matches_reference(name):
    from pyloki_gb300.scheme import MiddleOutScheme

    d = load_golden(name)
    if "final_leaves" not in d:
        pytest.skip("fixture stores no final leaves")
    cfg = _cfg(d, name)
    nseg = cfg.nsamps // cfg.bseg_ffa
    sc = MiddleOutScheme(nseg, int(d["ref_seg"]), cfg.tseg_ffa, 1)
    rep = chebyshev.report_batch(d["final_leaves"], sc.get_report_coord(bool(d["moving"])))
    np.testing.assert_allclose(rep, d["report"], rtol=1e-12, atol=0)


def test_transform_matrix_identities():
    # the same domain maps coefficients to themselves; R and S are inverses
    c = chebyshev.transform_matrix(4, 1.5, 2.0, 1.5, 2.0)
    np.testing.assert_allclose(c, np.eye(5), atol=1e-15)
    np.testing.assert_allclose(chebyshev.conn_matrix_s(5) @ chebyshev.conn_matrix_r(5),
                               np.eye(6), atol=1e-14)

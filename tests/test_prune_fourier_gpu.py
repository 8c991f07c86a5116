"""Enumerate-prune over Fourier-domain folds (use_fourier=True, the
reference's default) against runs of the pyloki reference.

The tree logic (branch, resolve, threshold, overflow, transform, backtracks)
is the exact path of the real-fold tree; only the fold arithmetic differs:
the complex64 phasor rotation and the irfft before scoring are evaluated
with CUDA's float32 sincos and summation order, so scores and folds are
compared to a float32 tolerance while the integer results and the FP64
leaves are compared as in the real-fold tests.
"""

from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import load_golden

pytestmark = pytest.mark.gpu
CASES = ["prune_taylor_fourier", "prune_cheby_fourier", "prune_circ_fourier"]
TOL_SCORE = 2e-5  # relative
TOL_FOLD = 2e-5   # of the row's largest magnitude


def _leaves_close(got, ref, what, circular):
    if not circular:
        np.testing.assert_allclose(got, ref, rtol=1e-13, atol=0, err_msg=what)
        return
    # circular propagation calls cos/sin (CUDA vs numpy in the last bit), and
    # its secular terms cancel: 1e-9 of the largest magnitude of each column
    scale = np.abs(ref).max(axis=0, keepdims=True)
    assert np.all(np.abs(got - ref) <= 1e-9 * scale), what


def _fold_err(got, ref):
    g = got.reshape(got.shape[0], -1)
    r = ref.reshape(ref.shape[0], -1)
    scale = np.abs(r).max(axis=1)
    scale[scale == 0] = 1.0
    return float((np.abs(g - r).max(axis=1) / scale).max()) if len(r) else 0.0


@pytest.mark.parametrize("name", CASES)
def test_fourier_prune_levels_match_reference(cuda_device, name):
    from pyloki_gb300.config import PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.prune import Pruning
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=True, bseg_ffa=int(d["bseg_ffa"]),
        prune_poly_order=int(d["poly_order"]), branch_max=int(d["branch_max"]),
        p_orb_min=float(d["p_orb_min"]))
    circ = int(d["poly_order"]) == 5
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device)
    dyp.initialize()
    dyp.execute()
    assert _fold_err(dyp.fold.cpu().numpy(), d["fold_ffa"]) <= TOL_FOLD
    prn = Pruning(dyp, d["thresholds"], max_sugg=int(d["max_sugg"]),
                  batch_size=int(d["batch_size"]), poly_basis=str(d["basis"]),
                  use_moving_grid=bool(d["moving"]))
    prn.initialize(int(d["ref_seg"]))
    wt = prn.world_tree
    _leaves_close(wt.leaves.cpu().numpy(), d["seed_leaves"], "seed leaves", circ)
    np.testing.assert_allclose(wt.scores.cpu().numpy(), d["seed_scores"], rtol=TOL_SCORE)
    nparams = prn.nparams_ffa
    for lvl in range(1, int(d["levels_done"]) + 1):
        prn.execute_iter()
        st = prn.pstats[-1]
        np.testing.assert_array_equal(
            [st.n_branches, st.n_leaves, st.n_leaves_phy, st.n_leaves_surv],
            d[f"stats_{lvl}"], err_msg=f"stats level {lvl}")
        wt = prn.world_tree
        np.testing.assert_allclose(wt.scores.cpu().numpy(), d[f"scores_{lvl}"],
                                   rtol=TOL_SCORE, err_msg=f"scores level {lvl}")
        if f"leaves_{lvl}" in d:
            _leaves_close(wt.leaves.cpu().numpy(), d[f"leaves_{lvl}"], f"leaves level {lvl}",
                          circ)
            bt = wt.backtracks.cpu().numpy()
            got = np.concatenate([bt[:, : nparams + 1], bt[:, -1:]], axis=1)
            np.testing.assert_array_equal(got, d[f"bt_{lvl}"], err_msg=f"bt level {lvl}")
        if f"folds_{lvl}" in d:
            assert _fold_err(wt.folds.cpu().numpy(), d[f"folds_{lvl}"]) <= TOL_FOLD
    prn._do_ascend()
    wt = prn.world_tree
    np.testing.assert_allclose(wt.scores.cpu().numpy(), d["asc_scores"], rtol=TOL_SCORE)
    np.testing.assert_allclose(wt.scores_ep.cpu().numpy(), d["asc_scores_ep"], rtol=TOL_SCORE)
    if "asc_folds" in d:
        assert _fold_err(wt.folds.cpu().numpy(), d["asc_folds"]) <= TOL_FOLD

"""Reduced-precision fold storage and FP64 candidate re-scoring on the GPU.

bfloat16 storage is checked bit for bit against the oracle applied to the
stored values: every stored level must equal the oracle's float32 shift-add of
the previous stored (bfloat16) level, rounded to bfloat16 (nearest even), and
the fused / banded searches must equal the oracle's float32 final level and
scoring of the stored penultimate level. The S/N error of bfloat16 storage is
then measured against the FP64 oracle, and the FP64 re-scoring kernel is
checked against the FP64 oracle to summation-order tolerance.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.conftest import cfg_from_golden, load_golden
from tests.test_ffa_gpu import _series

pytestmark = pytest.mark.gpu
FFA_CASES = ["ffa_freq", "ffa_accel", "ffa_jerk"]

# bfloat16 storage rounds every stored sum to 8 significant bits, so the S/N
# of a bfloat16 search carries an error of order 1e-2 against FP64 (0.096 at
# most, median about 0.006, on the 2^18 accel search below). The 1e-3 bound
# is met by re-scoring the retained candidates in FP64 (RESCORE_REL_TOL).
BF16_SNR_ABS_TOL = 0.25
BF16_SNR_REL_TOL = 2e-2  # |err| / max(|S/N_fp64|, 1)
# FP64 re-scoring differs from the FP64 oracle only by summation order.
RESCORE_REL_TOL = 1e-9


def _level(cfg, lvl, fold_in):
    """Oracle float32 shift-add of one level from a float32 copy of the input."""
    return O.ffa_level(cfg, lvl, np.ascontiguousarray(fold_in, np.float32))


def _bf16(x: np.ndarray) -> np.ndarray:
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(torch.bfloat16).float().numpy()


@pytest.mark.parametrize("name", FFA_CASES)
def test_bf16_levels_bit_exact_vs_rounded_oracle(cuda_device, name):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = cfg_from_golden(d)
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device, storage="bf16")
    dyp.initialize()
    assert dyp.fold.dtype == torch.bfloat16
    prev = dyp.fold.float().cpu().numpy()
    np.testing.assert_array_equal(prev, _bf16(d["fold_0"]))
    for lvl in range(1, cfg.niters_ffa + 1):
        dyp._execute_iter()
        got = dyp.fold.float().cpu().numpy()
        want = _bf16(_level(cfg, lvl, prev))
        np.testing.assert_array_equal(got, want.reshape(got.shape), err_msg=f"level {lvl}")
        prev = got
    np.testing.assert_array_equal(dyp.get_fold_norm().cpu().numpy(), O.fold_norm(prev[0]))


@pytest.mark.parametrize("name", FFA_CASES)
@pytest.mark.parametrize("final", ["level", "banded", "tiled"])
def test_bf16_search_bit_exact_vs_oracle_on_stored_levels(cuda_device, name, final):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = cfg_from_golden(d)
    w = np.asarray(cfg.score_widths)
    if final == "tiled" and not (cfg.nbins == 64 and np.array_equal(w, 2 ** np.arange(len(w)))):
        pytest.skip("50 bins and widths 1, 2, 3, 4, 6, 9: not a tiled configuration")
    ts = TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp)
    mat = DynamicProgramming(ts, cfg, device=cuda_device, storage="bf16")
    mat.initialize()
    for _ in range(cfg.niters_ffa - 1):
        mat._execute_iter()
    pen = mat.fold.float().cpu().numpy()
    fin = _level(cfg, cfg.niters_ffa, pen)
    want = O.boxcar_snr(O.fold_norm(fin[0]), cfg.score_widths)
    dyp = DynamicProgramming(ts, cfg, device=cuda_device, storage="bf16")
    dyp.initialize()
    got = dyp.search(final=final, band_bytes=4096).cpu().numpy()
    np.testing.assert_array_equal(got, want.reshape(got.shape))


@pytest.mark.parametrize("storage", ["f32", "bf16"])
@pytest.mark.parametrize("name", FFA_CASES)
def test_rescore_matches_fp64_oracle(cuda_device, name, storage):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden(name)
    cfg = cfg_from_golden(d)
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device, storage=storage)
    dyp.initialize()
    nq = int(np.prod(cfg.get_param_grid_count(cfg.niters_ffa)))
    cand = np.unique(np.r_[0, nq - 1, np.random.default_rng(1).integers(0, nq, 40)])
    snr, prof = dyp.rescore(cand, return_profiles=True)
    ref_prof = O.ffa_trials(d["ts_e"], d["ts_v"], cfg, cand, f64=True)
    np.testing.assert_allclose(prof.cpu().numpy(), ref_prof, rtol=RESCORE_REL_TOL, atol=1e-9)
    ref = O.boxcar_snr_f64(ref_prof, cfg.score_widths)
    np.testing.assert_allclose(snr.cpu().numpy(), ref, rtol=RESCORE_REL_TOL, atol=1e-9)
    # the f32 fixture S/N agrees with FP64 to float32 rounding
    np.testing.assert_allclose(d["snrs"].reshape(nq, -1)[cand], ref, rtol=1e-4, atol=1e-4)
    # every level as the candidates' level (rescore is not tied to the last one)
    lvl = max(1, cfg.niters_ffa - 1)
    nq1 = int(np.prod(cfg.get_param_grid_count(lvl)))
    c1 = np.arange(0, nq1, max(1, nq1 // 17))
    got1 = dyp.rescore(c1, level=lvl, seg=1).cpu().numpy()
    ref1 = O.boxcar_snr_f64(O.ffa_trials(d["ts_e"], d["ts_v"], cfg, c1, level=lvl, seg=1,
                                         f64=True), cfg.score_widths)
    np.testing.assert_allclose(got1, ref1, rtol=RESCORE_REL_TOL, atol=1e-9)
    # one segment per candidate
    segs = np.arange(len(c1)) % 2
    got2 = dyp.rescore(c1, level=lvl, seg=segs).cpu().numpy()
    np.testing.assert_allclose(got2[segs == 1], ref1[segs == 1], rtol=RESCORE_REL_TOL, atol=1e-9)
    ref0 = O.boxcar_snr_f64(O.ffa_trials(d["ts_e"], d["ts_v"], cfg, c1[segs == 0], level=lvl,
                                         seg=0, f64=True), cfg.score_widths)
    np.testing.assert_allclose(got2[segs == 0], ref0, rtol=RESCORE_REL_TOL, atol=1e-9)


def test_rescore_rejects_out_of_range_candidates(cuda_device):
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    d = load_golden("ffa_accel")
    cfg = cfg_from_golden(d)
    dyp = DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                             device=cuda_device, storage="bf16")
    dyp.initialize()
    nq = int(np.prod(cfg.get_param_grid_count(cfg.niters_ffa)))
    snr = dyp.rescore([-1, nq, 0]).cpu().numpy()
    assert np.isnan(snr[:2]).all() and np.isfinite(snr[2]).all()
    # a segment without all its level-0 segments is a NaN row, not an access
    snr = dyp.rescore([0, 0, 0], seg=[0, 1, -1]).cpu().numpy()
    assert np.isfinite(snr[0]).all() and np.isnan(snr[1:]).all()
    with pytest.raises(RuntimeError):  # no series on the device yet
        DynamicProgramming(TimeSeries(d["ts_e"], d["ts_v"], cfg.tsamp), cfg,
                           device=cuda_device).rescore([0])


def test_bf16_snr_error_vs_fp64_accel_search(cuda_device):
    """Banded accel search at 2^18 samples with bfloat16 storage: the S/N of
    sampled trials and of the top candidates against the FP64 oracle, and the
    top candidates re-scored in FP64 on the GPU."""
    from pyloki_gb300.config import ParamLimits, PulsarSearchConfig
    from pyloki_gb300.ffa import DynamicProgramming
    from pyloki_gb300.timeseries import TimeSeries

    n = 2**18
    cfg = PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
                             param_limits=ParamLimits.from_taylor((100.0, 140.0),
                                                                  accel=(-2000.0, 2000.0)).limits,
                             ducy_max=0.25, wtsp=2.0, use_fourier=False)
    ts_e, ts_v = _series(n, cfg.tsamp, 123.4, 0.4, 6, accel=700.0)
    ts = TimeSeries(ts_e, ts_v, cfg.tsamp)
    dyp = DynamicProgramming(ts, cfg, device=cuda_device, storage="bf16")
    snrs = dyp.search(banded=True, band_bytes=1 << 20)
    flat = snrs.reshape(-1, snrs.shape[-1])
    top = torch.topk(flat.amax(dim=1), 16).indices
    rng = np.random.default_rng(0)
    pick = np.unique(np.r_[top.cpu().numpy(), rng.integers(0, flat.shape[0], 300)])
    ref = O.boxcar_snr_f64(O.ffa_trials(ts_e, ts_v, cfg, pick, f64=True), cfg.score_widths)
    err = np.abs(flat.cpu().numpy()[pick].astype(np.float64) - ref)
    assert err.max() < BF16_SNR_ABS_TOL, err.max()
    assert (err / np.maximum(np.abs(ref), 1.0)).max() < BF16_SNR_REL_TOL
    resc = dyp.rescore(torch.from_numpy(pick)).cpu().numpy()
    np.testing.assert_allclose(resc, ref, rtol=RESCORE_REL_TOL, atol=1e-9)
    # the best trial is the same as with float32 storage
    f32 = DynamicProgramming(ts, cfg, device=cuda_device).search(banded=True, band_bytes=1 << 20)
    assert int(torch.argmax(f32.reshape(-1))) // flat.shape[1] == int(
        torch.argmax(flat.reshape(-1))) // flat.shape[1]

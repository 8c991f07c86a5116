"""Injection generator on the GPU against the reference's own outputs
(``tests/golden/pulse_*.npz``, pyloki's ``PulseSignalConfig.generate`` run
with a seeded generator) and the oracle.

Bit-exact: proper times of the Taylor model, the template from given proper
times, the emitted series from given noise and scales. Within stated
tolerances: proper times of the models that call ``sin``/``cos``/``atan``/
``pow`` (the device functions may differ from the host's libm in the last
ulp), the calibration (the device takes the off-pulse standard deviation in
float64 where numpy sums float32 pairwise), and everything downstream of the
exact folds (the reference's folds are float32 running sums).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import pulse_oracle as O

pytestmark = pytest.mark.gpu

CASES = sorted((Path(__file__).parent / "golden").glob("pulse_*.npz"))
IDS = [p.stem for p in CASES]
PT_ATOL = 1e-15       # s; proper times of the libm-based models (t <= 0.3 s)
SCALE_RTOL = 1e-5     # calibrated scales from float32 folds
SERIES_RTOL = 2e-5    # emitted samples downstream of the exact folds


def _cfg(c, **kw):
    from pyloki_gb300.pulse import PulseSignalConfig

    return PulseSignalConfig(period=float(c["period"]), dt=float(c["dt"]),
                             nsamps=int(c["nsamps"]), snr=float(c["snr"]),
                             ducy=float(c["ducy"]), mod_type=str(c["kind"]),
                             mod_kwargs=dict(c["params"]), **kw)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_template_and_proper_time(cuda_device, path):
    c = O.load_case(path)
    tm, pt = _cfg(c).template(str(c["shape"]), float(c["phi0"]), device=cuda_device,
                              return_proper_time=True)
    pt, tm = pt.cpu().numpy(), tm.cpu().numpy()
    if str(c["kind"]) == "derivative":
        np.testing.assert_array_equal(pt, c["proper_time"])
        np.testing.assert_array_equal(tm, c["template"])
    else:
        np.testing.assert_allclose(pt, c["proper_time"], rtol=0, atol=PT_ATOL)
        np.testing.assert_allclose(tm, c["template"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_template_from_reference_proper_times_bit_exact(cuda_device, path):
    from pyloki_gb300.pulse import generate_pulse_template

    c = O.load_case(path)
    tm = generate_pulse_template(c["proper_time"], float(c["dt"]), float(c["period"]), c["lut"],
                                 device=cuda_device)
    np.testing.assert_array_equal(tm.cpu().numpy(), c["template"])


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_calibration_on_reference_folds(cuda_device, path):
    from pyloki_gb300.pulse import _Batch

    c = O.load_case(path)
    b = _Batch([_cfg(c)], str(c["shape"]), float(c["phi0"]), 0, cuda_device)
    folds = torch.from_numpy(c["folds"].astype(np.float64))[None].to(cuda_device)
    out = b.calibrate(folds, 5, 1e-2).cpu().numpy()[0]
    np.testing.assert_allclose(out[0], float(c["noise_scale"]), rtol=1e-6)
    np.testing.assert_allclose(out[2], float(c["snr_template"]), rtol=1e-6)
    np.testing.assert_allclose(out[1], float(c["scale"]), rtol=SCALE_RTOL)
    # the oracle on the same folds (numpy's float32 std) lands on the same values
    ns, scale, snr_t, _ = O.calibrate(c["folds"][0], c["folds"][1], c["folds"][2],
                                      float(c["snr"]), float(c["ducy"]), float(c["phi0"]))
    np.testing.assert_allclose(out[1], scale, rtol=SCALE_RTOL)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_emit_with_reference_noise_and_scales(cuda_device, path):
    from pyloki_gb300.pulse import _Batch

    c = O.load_case(path)
    b = _Batch([_cfg(c)], str(c["shape"]), float(c["phi0"]), 0, cuda_device)
    scales = torch.tensor([[float(c["noise_scale"]), float(c["scale"]), 0.0, 0.0]],
                          dtype=torch.float64, device=cuda_device)
    noise = torch.from_numpy(c["noise"])[None].to(cuda_device)
    ts_e, ts_v = b.emit(scales, noise)
    np.testing.assert_array_equal(ts_v.cpu().numpy()[0], c["ts_v"])
    if str(c["kind"]) == "derivative":
        np.testing.assert_array_equal(ts_e.cpu().numpy()[0], c["ts_e"])
    else:
        np.testing.assert_allclose(ts_e.cpu().numpy()[0], c["ts_e"], rtol=0, atol=1e-5)


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_generate_with_reference_noise(cuda_device, path):
    c = O.load_case(path)
    ts = _cfg(c).generate(str(c["shape"]), float(c["phi0"]), noise=c["noise"],
                          device=cuda_device)
    e = ts.ts_e.cpu().numpy()
    scale = np.abs(c["ts_e"]).max()
    np.testing.assert_allclose(e, c["ts_e"], rtol=0, atol=SERIES_RTOL * scale)
    np.testing.assert_allclose(ts.ts_v.cpu().numpy(), c["ts_v"], rtol=1e-6)


def test_folds_equal_oracle_exact_sums(cuda_device):
    from pyloki_gb300.pulse import PulseSignalConfig, generate_injections

    c = O.load_case(CASES[0])
    cfg = PulseSignalConfig(period=float(c["period"]), dt=float(c["dt"]), nsamps=2**16,
                            snr=12.0, ducy=0.08, mod_kwargs={"acc": 12.0})
    rng = np.random.default_rng(0)
    noise = rng.standard_normal(2**16, dtype=np.float32)
    b = generate_injections([cfg], noise=noise, device=cuda_device)
    o = O.generate(cfg.period, cfg.dt, cfg.nsamps, 12.0, 0.08, noise, kind="derivative",
                   params={"acc": 12.0}, exact_folds=True)
    f = b.folds.cpu().numpy()[0][:, :cfg.fold_bins_ideal]
    # fixed-point sums: 2^-33 per sample at most
    np.testing.assert_allclose(f[0], o["folds"][0].astype(np.float64), rtol=0, atol=2e-5)
    np.testing.assert_array_equal(f[1], o["folds"][1])
    np.testing.assert_allclose(f[2], o["folds"][2].astype(np.float64), rtol=0, atol=2e-5)


def test_batch_is_deterministic_and_row_zero_is_single(cuda_device):
    from pyloki_gb300.pulse import PulseSignalConfig, generate_injections

    rng = np.random.default_rng(5)
    cfgs = [PulseSignalConfig(period=float(p), dt=64e-6, nsamps=2**15, snr=float(s),
                              ducy=float(d), mod_kwargs={"acc": float(a)})
            for p, s, d, a in zip(rng.uniform(2e-3, 2e-2, 8), rng.uniform(8, 30, 8),
                                  rng.uniform(0.03, 0.3, 8), rng.uniform(-50, 50, 8))]
    shapes = ["gaussian", "von_mises", "boxcar", "gaussian"] * 2
    phis = rng.uniform(0, 1, 8)
    a = generate_injections(cfgs, shapes, phis, seed=11, device=cuda_device)
    a2 = generate_injections(cfgs, shapes, phis, seed=11, device=cuda_device)
    assert torch.equal(a.ts_e, a2.ts_e) and torch.equal(a.scales, a2.scales)
    assert torch.equal(a.folds, a2.folds)
    one = cfgs[0].generate(shapes[0], float(phis[0]), seed=11, device=cuda_device)
    assert torch.equal(one.ts_e, a.ts_e[0])
    other = generate_injections(cfgs[:1], shapes[:1], phis[:1], seed=12, device=cuda_device)
    assert not torch.equal(a.ts_e[0], other.ts_e[0])


def test_calibrated_snr_reaches_target(cuda_device):
    from pyloki_gb300.pulse import PulseSignalConfig, generate_injections

    cfgs = [PulseSignalConfig(period=p, dt=64e-6, nsamps=2**18, snr=s, ducy=0.1)
            for p, s in ((3e-3, 10.0), (7e-3, 20.0), (1.3e-2, 40.0), (2.1e-2, 15.0))]
    b = generate_injections(cfgs, max_iter=40, seed=1, device=cuda_device)
    meas = b.scales[:, 3].cpu().numpy()
    np.testing.assert_allclose(meas, [c.snr for c in cfgs], atol=1e-2)
    # the folded S/N of the emitted series at the true period is that S/N:
    # fold ts_e, ts_v on the host and score with the oracle's boxcar
    for i, c in enumerate(cfgs):
        pt = c.proper_time
        bins = O.phase_bins(pt, 1.0 / c.period, c.fold_bins_ideal)
        e = np.bincount(bins, b.ts_e[i].cpu().numpy().astype(np.float64), c.fold_bins_ideal)
        v = np.bincount(bins, b.ts_v[i].cpu().numpy().astype(np.float64), c.fold_bins_ideal)
        got = float(O.boxcar_max_f32((e / np.sqrt(v)).astype(np.float32)))
        assert abs(got - c.snr) < 0.05 * c.snr


def test_noise_statistics(cuda_device):
    from pyloki_gb300.pulse import PulseSignalConfig

    cfg = PulseSignalConfig(period=5e-3, dt=64e-6, nsamps=2**20, snr=50.0, ducy=0.1)
    ts = cfg.generate_noise(seed=3, device=cuda_device)
    std = np.sqrt(cfg.nsamps * cfg.ducy) / cfg.snr / cfg.tol_bins
    x = ts.ts_e.cpu().numpy().astype(np.float64) / np.float32(std)
    n = x.size
    assert abs(x.mean()) < 5 / np.sqrt(n)
    assert abs(x.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    assert np.corrcoef(x[:-1], x[1:])[0, 1] < 5 / np.sqrt(n)
    assert np.all(ts.ts_v.cpu().numpy() == np.float32(std) * np.float32(std))


def test_table_modulation_for_any_model(cuda_device):
    """A model with only a host ``generate`` goes through a proper-time table."""
    from pyloki_gb300 import modulate
    from pyloki_gb300.pulse import PulseSignalConfig

    class Wobble:
        def __init__(self, amp: float = 1e-4) -> None:
            self.amp = amp

        def generate(self, t, t_ref=0.0):
            return t - self.amp * np.sin(3.0 * (t - t_ref)) ** 2

    modulate.type_to_mods["wobble"] = Wobble
    try:
        cfg = PulseSignalConfig(period=4e-3, dt=64e-6, nsamps=2**14, snr=12.0,
                                mod_type="wobble", mod_kwargs={"amp": 2e-4})
        tm, pt = cfg.template(device=cuda_device, return_proper_time=True)
        np.testing.assert_array_equal(pt.cpu().numpy(), cfg.proper_time)
        lut = O.cdf_lut("gaussian", 0.1, 0.5, 4096)
        np.testing.assert_array_equal(tm.cpu().numpy(),
                                      O.template(cfg.proper_time, cfg.dt, cfg.period, lut))
        ts = cfg.generate(seed=2, device=cuda_device)
        assert torch.isfinite(ts.ts_e).all()
    finally:
        del modulate.type_to_mods["wobble"]


def test_apply_path_equals_regenerated_series(cuda_device):
    """generate_injections scales the stored noise and template in place;
    regenerating both from the seeds with the same scales gives the same bits."""
    from pyloki_gb300.pulse import PulseSignalConfig, _Batch, generate_injections

    cfgs = [PulseSignalConfig(period=p, dt=64e-6, nsamps=2**16 + 3, snr=12.0, ducy=0.1,
                              mod_kwargs={"acc": a})
            for p, a in ((3e-3, 5.0), (9e-3, -20.0), (2.2e-2, 40.0))]
    b = generate_injections(cfgs, "von_mises", 0.3, seed=21, device=cuda_device)
    again = _Batch(cfgs, "von_mises", 0.3, 21, cuda_device)
    ts_e, ts_v = again.emit(b.scales, None)
    assert torch.equal(ts_e, b.ts_e) and torch.equal(ts_v, b.ts_v)


@pytest.mark.parametrize("shift", [0.0, 0.01 * 299792458.0])
def test_long_template_bit_exact(cuda_device, shift):
    """2^20 samples (t up to 67 s, tens of thousands of turns): the exact
    remainder of the phase, and the negative proper times of the first samples
    (the acceleration delay at t = 0, more of them with a 10 ms shift) that
    take the reference's fmod route."""
    from pyloki_gb300.pulse import PulseSignalConfig

    cfg = PulseSignalConfig(period=2.345e-3, dt=64e-6, nsamps=2**20, snr=10.0, ducy=0.05,
                            mod_kwargs={"shift": shift, "acc": 33.0, "jerk": -0.02})
    tm, pt = cfg.template("gaussian", 0.7, device=cuda_device, return_proper_time=True)
    ref_pt = O.proper_time("derivative", {"shift": shift, "acc": 33.0, "jerk": -0.02},
                           cfg.nsamps, cfg.dt, cfg.mod_tref)
    np.testing.assert_array_equal(pt.cpu().numpy(), ref_pt)
    assert (ref_pt < 0).any()  # both routes of the remainder run
    lut = O.cdf_lut("gaussian", 0.05, 0.7, max(4096, int(100 / 0.05)))
    np.testing.assert_array_equal(tm.cpu().numpy(), O.template(ref_pt, cfg.dt, cfg.period, lut))

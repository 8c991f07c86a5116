"""Host side of the injection generator: the modulation models reproduce the
reference's proper times (fixtures of ``PulseSignalConfig.proper_time``),
the CDF tables equal the reference's, the device constants are what the
kernel reads, and bad arguments fail before any kernel runs."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import pulse_oracle as O

CASES = sorted((Path(__file__).parent / "golden").glob("pulse_*.npz"))


def _cfg(c, **kw):
    from pyloki_gb300.pulse import PulseSignalConfig

    return PulseSignalConfig(period=float(c["period"]), dt=float(c["dt"]),
                             nsamps=int(c["nsamps"]), snr=float(c["snr"]),
                             ducy=float(c["ducy"]), mod_type=str(c["kind"]),
                             mod_kwargs=dict(c["params"]), **kw)


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_host_proper_time_and_lut_equal_reference(path):
    from pyloki_gb300.pulse import build_cdf_lut

    c = O.load_case(path)
    cfg = _cfg(c)
    assert cfg.mod_tref == float(c["t_ref"])
    assert cfg.fold_bins_ideal == int(c["nbins"])
    np.testing.assert_array_equal(cfg.proper_time, c["proper_time"])
    ngrid = max(4096, int(100 / float(c["ducy"])))
    np.testing.assert_array_equal(
        build_cdf_lut(str(c["shape"]), float(c["ducy"]), float(c["phi0"]), ngrid), c["lut"])


def test_encoded_constants():
    from pyloki_gb300 import _lib
    from pyloki_gb300.modulate import (CircularModulating, DerivativeModulating,
                                       DerivativeSeriesModulating, KeplerianModulating)

    m = DerivativeModulating(shift=1.0, vel=2.0, acc=3.0, jerk=4.0, snap=5.0).encode(7.0)
    assert m.kind == _lib.MOD_KINDS["derivative"] and m.t_ref == 7.0
    assert list(m.c)[:5] == [1.0, 2.0, 3.0, 4.0, 5.0]
    s = DerivativeSeriesModulating(coeffs=np.array([1.0, 2.0, 6.0, 24.0])).encode(0.0)
    assert s.ncoeff == 4 and list(s.c)[:4] == [1.0, 2.0, 3.0, 4.0]  # d^(k) / k!
    c = CircularModulating(p_orb=100.0, psi=0.5, x_orb=2.0).encode(1.0)
    assert list(c.c)[:3] == [2.0, 2 * np.pi / 100.0, 0.5]
    k = KeplerianModulating(p_orb=10.0, ecc=-0.5, phi=0.1, a=3.0, om=0.2, inc=0.3).encode(0.0)
    assert k.c[1] == 0.5 and k.c[3] == 3.0 * 0.75 and k.c[6] == np.sqrt(1.5 / 0.5)
    with pytest.raises(ValueError):
        DerivativeSeriesModulating(coeffs=np.ones(17)).encode(0.0)


def test_circular_from_masses_and_derivative_round_trip():
    from pyloki_gb300.modulate import CircularModulating, DerivativeModulating

    c = CircularModulating(p_orb=3600.0, psi=0.4, m_c=0.3)
    assert c.x_orb > 0
    d = c.to_derivatives()
    back = DerivativeModulating(acc=d["acc"], jerk=d["jerk"], snap=d["snap"]).to_circular()
    assert np.isclose(back["p_orb"], 3600.0) and np.isclose(back["x_orb"], c.x_orb)
    assert np.isclose(back["psi"], 0.4)


def test_validation_before_any_kernel():
    from pyloki_gb300.pulse import PulseSignalConfig, _Batch, generate_injections

    a = PulseSignalConfig(period=5e-3, dt=64e-6, nsamps=4096)
    with pytest.raises(ValueError, match="same nsamps"):
        _Batch([a, PulseSignalConfig(period=5e-3, dt=64e-6, nsamps=2048)], "gaussian", 0.5,
               0, "cpu")
    with pytest.raises(ValueError, match="same dt"):
        generate_injections([a, PulseSignalConfig(period=5e-3, dt=32e-6, nsamps=4096)],
                            device="cpu")
    with pytest.raises(ValueError, match="Unknown shape"):
        _Batch([a], "sawtooth", 0.5, 0, "cpu")
    with pytest.raises(ValueError, match="2 shapes for 1 injections"):
        _Batch([a], ["gaussian", "boxcar"], 0.5, 0, "cpu")
    with pytest.raises(ValueError):
        _Batch([a, a], "gaussian", [0.1, 0.2, 0.3], 0, "cpu")
    with pytest.raises(ValueError, match="calibration bins"):
        _Batch([PulseSignalConfig(period=1.0, dt=64e-6, nsamps=4096)], "gaussian", 0.5, 0,
               "cpu").fold(None)
    with pytest.raises(ValueError, match="at least 4"):
        _Batch([PulseSignalConfig(period=2e-4, dt=64e-6, nsamps=4096)], "gaussian", 0.5, 0,
               "cpu").fold(None)
    with pytest.raises(ValueError, match="Duty cycle"):
        PulseSignalConfig(period=5e-3, dt=64e-6, ducy=1.5)
    with pytest.raises(ValueError, match="Unknown modulation"):
        PulseSignalConfig(period=5e-3, dt=64e-6, mod_type="spiral")


def test_per_injection_seeds_are_distinct_and_reproducible():
    from pyloki_gb300.pulse import _seeds

    a, b = _seeds(3, 16), _seeds(3, 16)
    assert np.array_equal(a, b) and len(set(a.tolist())) == 16
    assert not np.array_equal(a, _seeds(4, 16))
    assert _seeds(3, 1)[0] == a[0]  # a single generate(seed) is row 0 of a batch


def test_batched_cdf_tables_equal_single_builds():
    from pyloki_gb300.pulse import build_cdf_lut, cdf_tables

    rng = np.random.default_rng(2)
    keys = []
    for shape in ("gaussian", "von_mises", "boxcar"):
        for d, ph in zip(rng.uniform(0.01, 0.5, 12), rng.uniform(0, 1, 12)):
            keys.append((shape, float(d), float(ph), max(4096, int(100 / d))))
    tables = cdf_tables(keys)
    for k in keys:
        np.testing.assert_array_equal(tables[k], build_cdf_lut(k[0], k[1], k[2], k[3]))


def test_matched_filter_host_checks():
    from pyloki_gb300.scoring import MatchedFilter

    with pytest.raises(ValueError, match="must divide"):
        MatchedFilter([2, 6], 50, shift=4)
    with pytest.raises(ValueError, match="greater than 0"):
        MatchedFilter([2], 64, shift=0)
    with pytest.raises(ValueError, match="Unknown template"):
        MatchedFilter([2], 64, kind="sinc")
    mf = MatchedFilter([1, 3], 64, shift=2, kind="gaussian")
    assert mf.e_mat.shape == (64, 64) and np.allclose((mf.e_mat**2).sum(1), 1, atol=1e-5)

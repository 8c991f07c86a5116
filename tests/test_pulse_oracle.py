"""The generator oracle against the reference's own outputs: every fixture
(``tests/golden/pulse_*.npz``, made by running pyloki's
``PulseSignalConfig.generate`` with a seeded generator) is reproduced bit for
bit — proper times, CDF table, template, float32 folds, noise and signal
scales, and the emitted series."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import pulse_oracle as O

CASES = sorted((Path(__file__).parent / "golden").glob("pulse_*.npz"))


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_oracle_reproduces_reference_generate(path):
    c = O.load_case(path)
    o = O.generate(float(c["period"]), float(c["dt"]), int(c["nsamps"]), float(c["snr"]),
                   float(c["ducy"]), c["noise"], shape=str(c["shape"]), phi0=float(c["phi0"]),
                   kind=str(c["kind"]), params=c["params"], t_ref=float(c["t_ref"]))
    np.testing.assert_array_equal(o["proper_time"], c["proper_time"])
    np.testing.assert_array_equal(o["lut"], c["lut"])
    np.testing.assert_array_equal(o["template"], c["template"])
    np.testing.assert_array_equal(o["folds"], c["folds"])
    assert o["noise_scale"] == float(c["noise_scale"])
    assert o["snr_template"] == float(c["snr_template"])
    assert o["scale"] == float(c["scale"])
    np.testing.assert_array_equal(o["ts_e"], c["ts_e"])
    np.testing.assert_array_equal(o["ts_v"], c["ts_v"])


def test_fixtures_cover_every_modulation_and_shape():
    kinds = {str(O.load_case(p)["kind"]) for p in CASES}
    shapes = {str(O.load_case(p)["shape"]) for p in CASES}
    assert kinds == {"derivative", "derivative_series", "circular", "circular_t0", "keplerian"}
    assert shapes == {"gaussian", "von_mises", "boxcar"}


def test_calibration_reaches_target_snr():
    """On exact folds of a long series the calibrated S/N comes within tol
    (the damped Newton steps need more than the default five here)."""
    rng = np.random.default_rng(1)
    n = 2**16
    noise = rng.standard_normal(n, dtype=np.float32)
    o = O.generate(5.2e-3, 64e-6, n, 12.0, 0.1, noise, exact_folds=True, max_iter=30)
    assert abs(o["snr_measured"] - 12.0) < 1e-2


def test_off_pulse_window_wraps():
    m = O.off_pulse_mask(10, 0.3, 0.05)  # centre bin 0 (round half to even), 3 bins
    assert m.tolist() == [False, False, True, True, True, True, True, True, True, False]

"""Host logic of the batched search: length rounding, the tuner's choice,
memory limit and JSON persistence (no GPU: timings come from a model)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from pyloki_gb300.batch import Tuner, _peak_bytes, cfg3_lengths, pow2_length
from pyloki_gb300.config import ParamLimits, PulsarSearchConfig


def _cfg(n=2**15):
    return PulsarSearchConfig(nsamps=n, tsamp=64e-6, nbins=64, eta=1.0,
                              param_limits=ParamLimits.from_taylor(
                                  (100.0, 140.0), accel=(-2000.0, 2000.0)).limits,
                              ducy_max=0.25, wtsp=2.0, use_fourier=False, bseg_brute=4096)


def test_pow2_length():
    assert pow2_length(1) == 1
    assert pow2_length(2**20) == 2**20
    assert pow2_length(2**20 + 1) == 2**20
    assert pow2_length(2**21 - 1) == 2**20
    with pytest.raises(ValueError):
        pow2_length(0)


def test_cfg3_lengths_seeded_and_in_range():
    a = cfg3_lengths(256, 3)
    assert np.array_equal(a, cfg3_lengths(256, 3))
    assert a.min() >= 2**20 and a.max() <= 2**23
    assert {pow2_length(int(x)) for x in a} <= {2**20, 2**21, 2**22, 2**23}


def test_peak_bytes_grows_with_batch():
    cfg = _cfg()
    b = [_peak_bytes(cfg, c, 1 << 20, 4) for c in (1, 2, 4, 8)]
    assert all(x < y for x, y in zip(b, b[1:]))
    assert _peak_bytes(cfg, 4, 1 << 20, 2) < _peak_bytes(cfg, 4, 1 << 20, 4)


def test_tuner_picks_fastest_within_budget_and_persists(tmp_path):
    cfg = _cfg()
    calls = []

    def time_fn(chunk, band):
        calls.append((chunk, band))
        # per-series cost falls until chunk 4, then rises; the 32 MiB band is best
        per = {1: 10.0, 2: 6.0, 4: 4.0, 8: 5.0, 16: 9.0}[chunk]
        return chunk * per * (0.9 if band == 32 << 20 else 1.0)

    path = tmp_path / "tune.json"
    bands = (32 << 20, 96 << 20, 256 << 20)
    t = Tuner(path, band_choices=bands)
    dev = torch.device("cpu")
    big = _peak_bytes(cfg, 16, 256 << 20, 4)
    res = t.tune(cfg, "f32", dev, 16, big, time_fn)
    assert res.chunk == 4 and res.band_bytes == 32 << 20
    assert (16, 96 << 20) not in calls  # stopped once chunks got slower
    # a second tuner reads the file instead of timing again
    calls.clear()
    res2 = Tuner(path, band_choices=bands).tune(cfg, "f32", dev, 16, big, time_fn)
    assert calls == [] and (res2.chunk, res2.band_bytes) == (4, 32 << 20)
    # a memory budget below two series limits the chunk to one
    small = _peak_bytes(cfg, 1, 256 << 20, 2)
    res3 = Tuner(band_choices=bands).tune(cfg, "bf16", dev, 16, small, time_fn)
    assert res3.chunk == 1
    with pytest.raises(MemoryError):
        Tuner(band_choices=bands).tune(cfg, "f32", dev, 4, 1024, time_fn)

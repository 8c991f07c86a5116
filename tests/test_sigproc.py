"""SIGPROC .tim and PRESTO .dat/.inf files (the inputs of TimeSeries.from_tim,
io/timeseries.py:198-236): round trips through the package's writers,
8-bit and signed samples, and malformed files rejected with a message."""

from __future__ import annotations

import struct

import numpy as np
import pytest

from pyloki_gb300 import sigproc


def test_tim_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(1000).astype(np.float32)
    p = tmp_path / "a.tim"
    sigproc.write_tim(p, x, 6.4e-5, source_name="J0000+00", refdm=12.5, nsamples=1000)
    got, hdr = sigproc.read_tim(p)
    np.testing.assert_array_equal(got, x)
    assert hdr["tsamp"] == 6.4e-5 and hdr["source_name"] == "J0000+00"
    assert hdr["refdm"] == 12.5 and hdr["nbits"] == 32 and hdr["nsamples"] == 1000


def _raw_tim(path, nbits, data: bytes, signed=None):
    out = bytearray()
    for s in ("HEADER_START", "tsamp"):
        out += struct.pack("<i", len(s)) + s.encode()
        if s == "tsamp":
            out += struct.pack("<d", 1e-3)
    out += struct.pack("<i", 5) + b"nbits" + struct.pack("<i", nbits)
    if signed is not None:
        out += struct.pack("<i", 6) + b"signed" + bytes([signed])
    out += struct.pack("<i", 10) + b"HEADER_END" + data
    path.write_bytes(bytes(out))


def test_tim_8bit_unsigned_and_signed(tmp_path):
    raw = bytes([0, 1, 200, 255])
    _raw_tim(tmp_path / "u.tim", 8, raw)
    got, _ = sigproc.read_tim(tmp_path / "u.tim")
    np.testing.assert_array_equal(got, [0, 1, 200, 255])
    _raw_tim(tmp_path / "s.tim", 8, raw, signed=1)
    got, _ = sigproc.read_tim(tmp_path / "s.tim")
    np.testing.assert_array_equal(got, [0, 1, -56, -1])


def test_tim_rejects_malformed(tmp_path):
    p = tmp_path / "bad.tim"
    p.write_bytes(struct.pack("<i", 5) + b"HELLO")
    with pytest.raises(ValueError, match="HEADER_START"):
        sigproc.read_tim(p)
    out = bytearray(struct.pack("<i", 12) + b"HEADER_START")
    out += struct.pack("<i", 7) + b"bogus_k" + struct.pack("<i", 1)
    p.write_bytes(bytes(out))
    with pytest.raises(ValueError, match="unknown SIGPROC header keyword"):
        sigproc.read_tim(p)
    _raw_tim(p, 32, b"\x00\x00\x80")  # not whole float32 samples
    with pytest.raises(ValueError, match="whole"):
        sigproc.read_tim(p)
    _raw_tim(p, 12, b"")
    with pytest.raises(ValueError, match="nbits"):
        sigproc.read_tim(p)


def test_dat_round_trip_and_checks(tmp_path):
    rng = np.random.default_rng(2)
    x = rng.standard_normal(777).astype(np.float32)
    p = tmp_path / "b.dat"
    sigproc.write_dat(p, x, 1.28e-4, **{"Telescope used": "GB300"})
    got, info = sigproc.read_dat(p)
    np.testing.assert_array_equal(got, x)
    assert info["tsamp"] == 1.28e-4 and info["Telescope used"] == "GB300"
    (tmp_path / "b.inf").write_text(" Number of bins in the time series  =  5\n")
    with pytest.raises(ValueError, match="Width of each time series bin"):
        sigproc.read_dat(p)
    sigproc.write_dat(p, x, 1.28e-4)
    p.write_bytes(x[:-1].tobytes())
    with pytest.raises(ValueError, match="777 samples"):
        sigproc.read_dat(p)


def test_from_tim_rejects_unknown_type(tmp_path):
    from pyloki_gb300.timeseries import TimeSeries

    with pytest.raises(ValueError, match="Invalid tim type"):
        TimeSeries.from_tim(tmp_path / "x.fil", tim_type="fil")

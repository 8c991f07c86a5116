"""Time-series files read by ``TimeSeries.from_tim`` (``io/timeseries.py:198-236``).

The reference reads them through sigpyproc (``TimeSeries.from_tim`` /
``from_dat``); the formats are restated here from their public definitions:

- SIGPROC ``.tim``: a header of keyword records between ``HEADER_START`` and
  ``HEADER_END`` (every string an int32 length and its bytes; values int32,
  float64, a one-byte ``signed`` flag, or a string), then the samples
  (``nbits`` 32: float32; 16: uint16; 8: uint8, or int8 when ``signed``).
- PRESTO ``.dat`` + ``.inf``: raw little-endian float32 samples and a text
  file of ``description = value`` lines; the sampling time is the value of
  ``Width of each time series bin (sec)``.

``write_tim`` / ``write_dat`` write the same formats (test inputs, exported
series).
"""

from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

_STR_KEYS = {"source_name", "rawdatafile"}
_INT_KEYS = {"telescope_id", "machine_id", "data_type", "barycentric", "pulsarcentric",
             "nbits", "nsamples", "nchans", "nifs", "nbeams", "ibeam"}
_DOUBLE_KEYS = {"tstart", "tsamp", "fch1", "foff", "refdm", "az_start", "za_start",
                "src_raj", "src_dej", "period", "fchannel"}
_CHAR_KEYS = {"signed"}
_MARKERS = {"HEADER_START", "HEADER_END", "FREQUENCY_START", "FREQUENCY_END"}

INF_TSAMP = "Width of each time series bin (sec)"
INF_NSAMPS = "Number of bins in the time series"


def _read_str(buf: bytes, off: int) -> tuple[str, int]:
    if off + 4 > len(buf):
        msg = "truncated SIGPROC header"
        raise ValueError(msg)
    (n,) = struct.unpack_from("<i", buf, off)
    if n < 1 or n > 80 or off + 4 + n > len(buf):
        msg = f"bad SIGPROC header string length {n} at byte {off}"
        raise ValueError(msg)
    return buf[off + 4:off + 4 + n].decode("ascii", errors="strict"), off + 4 + n


def read_sigproc_header(buf: bytes) -> tuple[dict, int]:
    """Keyword values of a SIGPROC header and its length in bytes."""
    key, off = _read_str(buf, 0)
    if key != "HEADER_START":
        msg = "not a SIGPROC file: no HEADER_START"
        raise ValueError(msg)
    hdr: dict = {}
    while True:
        key, off = _read_str(buf, off)
        if key == "HEADER_END":
            return hdr, off
        if key in _MARKERS:
            continue
        if key in _STR_KEYS:
            hdr[key], off = _read_str(buf, off)
        elif key in _INT_KEYS:
            (hdr[key],) = struct.unpack_from("<i", buf, off)
            off += 4
        elif key in _DOUBLE_KEYS:
            (val,) = struct.unpack_from("<d", buf, off)
            off += 8
            if key == "fchannel":
                hdr.setdefault("fchannel", []).append(val)
            else:
                hdr[key] = val
        elif key in _CHAR_KEYS:
            hdr[key] = buf[off]
            off += 1
        else:
            msg = f"unknown SIGPROC header keyword {key!r}"
            raise ValueError(msg)


def read_tim(path) -> tuple[np.ndarray, dict]:
    """Samples (float32) and header of a SIGPROC time series."""
    buf = Path(path).read_bytes()
    hdr, off = read_sigproc_header(buf)
    if hdr.get("nchans", 1) != 1:
        msg = f"{path}: a time series has one channel, the header says {hdr['nchans']}"
        raise ValueError(msg)
    if "tsamp" not in hdr or not hdr["tsamp"] > 0:
        msg = f"{path}: missing or non-positive tsamp"
        raise ValueError(msg)
    nbits = hdr.get("nbits", 32)
    dtypes = {32: "<f4", 16: "<u2", 8: "<i1" if hdr.get("signed", 0) else "u1"}
    if nbits not in dtypes:
        msg = f"{path}: nbits {nbits} not supported (8, 16 or 32)"
        raise ValueError(msg)
    dt = np.dtype(dtypes[nbits])
    nbytes = len(buf) - off
    if nbytes % dt.itemsize:
        msg = f"{path}: {nbytes} data bytes are not whole {nbits}-bit samples"
        raise ValueError(msg)
    data = np.frombuffer(buf, dtype=dt, offset=off).astype(np.float32)
    if "nsamples" in hdr and hdr["nsamples"] not in (0, len(data)):
        msg = f"{path}: header nsamples {hdr['nsamples']} but {len(data)} samples"
        raise ValueError(msg)
    return data, hdr


def _write_str(out: bytearray, s: str) -> None:
    b = s.encode("ascii")
    out += struct.pack("<i", len(b)) + b


def write_tim(path, data, tsamp: float, **header) -> None:
    """Write a float32 SIGPROC time series (nbits 32, one channel)."""
    hdr = {"nbits": 32, "nchans": 1, "nifs": 1, "data_type": 2, "tsamp": float(tsamp),
           "tstart": 0.0, **header}
    out = bytearray()
    _write_str(out, "HEADER_START")
    for key, val in hdr.items():
        _write_str(out, key)
        if key in _STR_KEYS:
            _write_str(out, str(val))
        elif key in _INT_KEYS:
            out += struct.pack("<i", int(val))
        elif key in _DOUBLE_KEYS:
            out += struct.pack("<d", float(val))
        elif key in _CHAR_KEYS:
            out += struct.pack("<B", int(val))
        else:
            msg = f"unknown SIGPROC header keyword {key!r}"
            raise ValueError(msg)
    _write_str(out, "HEADER_END")
    out += np.ascontiguousarray(data, dtype="<f4").tobytes()
    Path(path).write_bytes(bytes(out))


def _inf_path(path) -> Path:
    p = Path(path)
    return p.with_suffix(".inf")


def read_inf(path) -> dict:
    """``description = value`` lines of a PRESTO .inf file."""
    info: dict = {}
    for line in _inf_path(path).read_text().splitlines():
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        info[k.strip()] = v.strip()
    return info


def read_dat(path) -> tuple[np.ndarray, dict]:
    """Samples (float32) and .inf values of a PRESTO time series."""
    info = read_inf(path)
    if INF_TSAMP not in info:
        msg = f"{_inf_path(path)}: no '{INF_TSAMP}' line"
        raise ValueError(msg)
    tsamp = float(info[INF_TSAMP])
    if not tsamp > 0:
        msg = f"{_inf_path(path)}: non-positive sampling time {tsamp}"
        raise ValueError(msg)
    raw = Path(path).read_bytes()
    if len(raw) % 4:
        msg = f"{path}: {len(raw)} bytes are not whole float32 samples"
        raise ValueError(msg)
    data = np.frombuffer(raw, dtype="<f4").astype(np.float32)
    if INF_NSAMPS in info and int(float(info[INF_NSAMPS])) != len(data):
        msg = f"{path}: .inf gives {info[INF_NSAMPS]} samples, the file holds {len(data)}"
        raise ValueError(msg)
    info["tsamp"] = tsamp
    return data, info


def write_dat(path, data, tsamp: float, **fields) -> None:
    """Write a PRESTO .dat (float32) and its .inf."""
    data = np.ascontiguousarray(data, dtype="<f4")
    Path(path).write_bytes(data.tobytes())
    lines = {" Data file name without suffix": Path(path).with_suffix("").name,
             " " + INF_NSAMPS: str(len(data)), " " + INF_TSAMP: repr(float(tsamp)),
             **{" " + k: str(v) for k, v in fields.items()}}
    _inf_path(path).write_text(
        "".join(f"{k:<40s}=  {v}\n" for k, v in lines.items()))


__all__ = ["read_dat", "read_inf", "read_sigproc_header", "read_tim", "write_dat",
           "write_tim"]

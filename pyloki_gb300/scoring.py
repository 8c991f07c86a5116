"""Boxcar S/N scoring on the GPU (``detection/scoring.py``).

``boxcar_snr_nd`` and ``snr_score_batch`` accept numpy arrays (copied to the
device and back, like a drop-in for the reference functions) or CUDA torch
tensors (kept on the device).
"""

from __future__ import annotations

import numpy as np
import torch

from pyloki_gb300 import _lib
from pyloki_gb300.config import generate_box_width_trials

__all__ = ["boxcar_snr_nd", "generate_box_width_trials", "snr_score_batch"]


def _to_device(data, device) -> tuple[torch.Tensor, bool]:
    if isinstance(data, torch.Tensor):
        return data.to(device=device, dtype=torch.float32).contiguous(), False
    arr = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
    return torch.from_numpy(arr).to(device), True


def boxcar_snr_nd(data, widths, stdnoise: float = 1.0, *, device=None):
    """S/N of normalised profiles ``(..., nbins)`` -> ``(..., nwidths)``
    (``detection/scoring.py:156-165``)."""
    lib = _lib.load()
    device = device or (data.device if isinstance(data, torch.Tensor) else "cuda")
    x, host = _to_device(data, device)
    nbins = x.shape[-1]
    widths = np.asarray(widths, dtype=np.int64)
    flat = x.reshape(-1, nbins)
    out = torch.empty((flat.shape[0], len(widths)), dtype=torch.float32, device=x.device)
    spec = _lib.score_spec(widths, nbins, stdnoise, mode=0)
    stream = torch.cuda.current_stream(x.device)
    _lib.check(lib.loki_boxcar_snr(_lib.ptr(flat), flat.shape[0], nbins, spec,
                                   _lib.ptr(out), _lib.stream_ptr(stream)))
    out = out.reshape(*x.shape[:-1], len(widths))
    return out.cpu().numpy() if host else out


def snr_score_batch(folds, widths, *, device=None):
    """Max-over-widths S/N of ``(n, 2, nbins)`` folds
    (``detection/scoring.py:249-282`` snr_score_batch_func)."""
    lib = _lib.load()
    device = device or (folds.device if isinstance(folds, torch.Tensor) else "cuda")
    x, host = _to_device(folds, device)
    n, _, nbins = x.shape
    out = torch.empty(n, dtype=torch.float32, device=x.device)
    spec = _lib.score_spec(widths, nbins, 1.0, mode=1)
    stream = torch.cuda.current_stream(x.device)
    _lib.check(lib.loki_snr_score_batch(_lib.ptr(x), n, nbins, spec, _lib.ptr(out),
                                        _lib.stream_ptr(stream)))
    return out.cpu().numpy() if host else out

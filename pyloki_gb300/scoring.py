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

__all__ = ["MatchedFilter", "boxcar_snr_nd", "generate_box_width_trials",
           "harmonic_summing_score", "kadane_circular_normalized", "snr_score_batch"]


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


# ---- alternative scorers (detection/scoring.py:295-755) ----------------------
# Constants of the interpolation tables (utils/maths.py:71-76).
CHI_SQ_RES, CHI_SQ_MAX, CHI_SQ_DF_MAX = 0.5, 300.0, 64
MINUS_LOGSF_RES, MAX_MINUS_LOGSF = 0.1, 400.0
_TABLES: dict = {}


def score_tables_host() -> tuple[np.ndarray, np.ndarray]:
    """-log sf of chi-square (rows df = 0..64, plus a zero row) and the normal
    ISF of exp(-x) (plus the last value repeated), as the reference builds
    them (utils/maths.py:55-77). The extra row and value keep the one-past-
    the-end reads of the interpolation inside the tables; the device wraps
    negative positions with the reference's table length."""
    from scipy import stats

    x = np.arange(0, CHI_SQ_MAX, CHI_SQ_RES)
    chi = np.zeros((CHI_SQ_DF_MAX + 2, len(x)))
    for i in range(1, CHI_SQ_DF_MAX + 1):
        chi[i] = -stats.chi2.logsf(x, i)
    isf = stats.norm.isf(np.exp(-np.arange(0, MAX_MINUS_LOGSF, MINUS_LOGSF_RES)))
    return chi, np.append(isf, isf[-1])


def _tables(device: torch.device):
    key = str(device)
    if key not in _TABLES:
        chi, isf = score_tables_host()
        _TABLES[key] = (torch.from_numpy(chi).to(device), torch.from_numpy(isf).to(device))
    return _TABLES[key]


def _normalise(arr: np.ndarray) -> np.ndarray:
    """Zero mean, unit energy (scoring.py:360-381)."""
    m = (arr - np.mean(arr)).astype(np.float32)
    norm = np.sqrt(np.dot(m, m))
    return m if norm == 0 else m / norm


def gen_boxcar_templates(widths, nbins: int) -> np.ndarray:
    """(scoring.py:384-409)"""
    t = np.zeros((len(widths), nbins), dtype=np.float32)
    for iw, w in enumerate(widths):
        t[iw, :w] = 1
        t[iw] = _normalise(t[iw])
    return t


def gen_gaussian_templates(widths, nbins: int) -> np.ndarray:
    """Gaussians of FWHM ``widths`` bins centred at nbins // 2 (scoring.py:412-441)."""
    t = np.zeros((len(widths), nbins), dtype=np.float32)
    for iw, w in enumerate(widths):
        sigma = w / (2 * np.sqrt(2 * np.log(2)))
        xmax = int(np.ceil(3.5 * sigma))
        xx = np.arange(-xmax, xmax + 1)
        data = np.exp(-(xx**2) / (2 * sigma**2))
        if nbins >= 2 * xmax + 1:
            t[iw, nbins // 2 - xmax:nbins // 2 + xmax + 1] = data
        else:
            start = xmax - nbins // 2
            t[iw, :nbins] = data[start:start + nbins]
        t[iw] = _normalise(t[iw])
    return t


def get_e_mat(templates: np.ndarray, shifts: np.ndarray) -> np.ndarray:
    """Every template at every multiple of its shift (scoring.py:444-470)."""
    ntemp, nbins = templates.shape
    rows = [np.roll(templates[i], j) for i in range(ntemp) for j in range(0, nbins, shifts[i])]
    return np.asarray(rows, dtype=np.float32)


class MatchedFilter:
    """Bank of mean-free, unit-power boxcar or Gaussian templates at every
    circular shift (``scoring.py:295-357``), scored on the GPU.

    The shift must divide ``nbins``: the reference sizes its bank as
    ``nbins // shift`` rows per template and overruns it otherwise."""

    def __init__(self, widths, nbins: int, shift: int = 1, kind: str = "boxcar") -> None:
        self.widths = np.asarray(widths, dtype=np.int64)
        self.nbins = int(nbins)
        self.kind = kind
        if kind == "boxcar":
            self.templates = gen_boxcar_templates(self.widths, self.nbins)
        elif kind == "gaussian":
            self.templates = gen_gaussian_templates(self.widths, self.nbins)
        else:
            msg = f"Unknown template shape: {kind}"
            raise ValueError(msg)
        if shift <= 0:
            msg = "Shift must be greater than 0."
            raise ValueError(msg)
        if self.nbins % shift:
            msg = f"shift {shift} must divide nbins {self.nbins}"
            raise ValueError(msg)
        self.shifts = np.full(self.ntemp, shift, dtype=np.int64)
        self.e_mat = get_e_mat(self.templates, self.shifts)
        self._dev: dict = {}

    @property
    def ntemp(self) -> int:
        return len(self.templates)

    def _device_bank(self, device):
        key = str(device)
        if key not in self._dev:
            inner = np.dot(self.e_mat, self.e_mat.T).astype(np.float32)  # host, as the reference
            self._dev[key] = (torch.from_numpy(self.e_mat).to(device),
                              torch.from_numpy(inner).to(device))
        return self._dev[key]

    def _run(self, norm_data, device, with_proj: bool, stdnoise: float = 1.0):
        device = device or (norm_data.device if isinstance(norm_data, torch.Tensor) else "cuda")
        x, host = _to_device(norm_data, device)
        flat = x.reshape(-1, self.nbins).contiguous()
        e, _ = self._device_bank(x.device)
        nfilt = e.shape[0]
        snr = torch.empty((flat.shape[0], self.ntemp), dtype=torch.float32, device=x.device)
        proj = (torch.empty((flat.shape[0], nfilt), dtype=torch.float32, device=x.device)
                if with_proj else None)
        _lib.check(_lib.load().loki_matched_filter(
            _lib.ptr(flat), flat.shape[0], self.nbins, _lib.ptr(e), nfilt,
            self.nbins // int(self.shifts[0]), float(stdnoise), _lib.ptr(snr), _lib.ptr(proj),
            _lib.stream_ptr(torch.cuda.current_stream(x.device))))
        return x, host, snr, proj

    def compute_snr(self, norm_data, stdnoise: float = 1.0, *, device=None):
        """Max projection per template, ``(..., nbins) -> (..., ntemp)``
        (``compute_snr_e_mat_2d``)."""
        x, host, snr, _ = self._run(norm_data, device, False, stdnoise)
        snr = snr.reshape(*x.shape[:-1], self.ntemp)
        return snr.cpu().numpy() if host else snr

    def compute_dot(self, folds, *, device=None):
        """``e_mat @ folds`` for folds ``(nbins,)`` or ``(nbins, nprof)``."""
        t = folds if isinstance(folds, torch.Tensor) else np.asarray(folds, np.float32)
        prof = t.T if t.ndim == 2 else t[None, :]
        if isinstance(prof, torch.Tensor):
            prof = prof.contiguous()
        _, host, _, proj = self._run(prof, device, True)
        proj = proj.T if t.ndim == 2 else proj[0]
        return proj.cpu().numpy() if host else proj.contiguous()

    def compute_fft(self, folds, *, device=None):
        """Max over the first nbins lags of the circular convolution of each
        profile (circularly padded to a power of two) with each template,
        ``(..., nbins) -> (..., ntemp)`` (``_compute_snr_fft``)."""
        device = device or (folds.device if isinstance(folds, torch.Tensor) else "cuda")
        x, host = _to_device(folds, device)
        flat = x.reshape(-1, self.nbins).contiguous()
        key = f"templates:{x.device}"
        if key not in self._dev:
            self._dev[key] = torch.from_numpy(self.templates).to(x.device)
        tm = self._dev[key]
        out = torch.empty((flat.shape[0], self.ntemp), dtype=torch.float32, device=x.device)
        _lib.check(_lib.load().loki_matched_filter_conv(
            _lib.ptr(flat), flat.shape[0], self.nbins, _lib.ptr(tm), self.ntemp, _lib.ptr(out),
            _lib.stream_ptr(torch.cuda.current_stream(x.device))))
        out = out.reshape(*x.shape[:-1], self.ntemp)
        return out.cpu().numpy() if host else out

    def compute_dot_double(self, folds, n_corr: int = 10, *, device=None):
        """Two-peak score per profile (``_compute_snr_double``)."""
        device = device or (folds.device if isinstance(folds, torch.Tensor) else "cuda")
        x, host = _to_device(folds, device)
        flat = x.reshape(-1, self.nbins).contiguous()
        e, inner = self._device_bank(x.device)
        chi, isf = _tables(x.device)
        out = torch.empty(flat.shape[0], dtype=torch.float32, device=x.device)
        _lib.check(_lib.load().loki_matched_filter_double(
            _lib.ptr(flat), flat.shape[0], self.nbins, _lib.ptr(e), e.shape[0],
            _lib.ptr(inner), int(n_corr), _lib.ptr(chi), chi.shape[1], CHI_SQ_RES, CHI_SQ_MAX,
            _lib.ptr(isf), isf.numel() - 1, MINUS_LOGSF_RES, MAX_MINUS_LOGSF, _lib.ptr(out),
            _lib.stream_ptr(torch.cuda.current_stream(x.device))))
        out = out.reshape(x.shape[:-1])
        return out.cpu().numpy() if host else out


def kadane_circular_normalized(norm_data, biases, *, device=None):
    """Best circular window per profile over the biases
    (``kadane_circular_normalized_1d``): (snr float64, width, start) arrays
    of shape ``norm_data.shape[:-1]``."""
    device = device or (norm_data.device if isinstance(norm_data, torch.Tensor) else "cuda")
    x, host = _to_device(norm_data, device)
    nb = x.shape[-1]
    flat = x.reshape(-1, nb).contiguous()
    b = torch.as_tensor(np.asarray(biases, np.float32)).to(x.device)
    n = flat.shape[0]
    snr = torch.empty(n, dtype=torch.float64, device=x.device)
    width = torch.empty(n, dtype=torch.int64, device=x.device)
    start = torch.empty(n, dtype=torch.int64, device=x.device)
    _lib.check(_lib.load().loki_kadane_circular(
        _lib.ptr(flat), n, nb, _lib.ptr(b), b.numel(), _lib.ptr(snr), _lib.ptr(width),
        _lib.ptr(start), _lib.stream_ptr(torch.cuda.current_stream(x.device))))
    res = [t.reshape(x.shape[:-1]) for t in (snr, width, start)]
    return tuple(t.cpu().numpy() for t in res) if host else tuple(res)


def harmonic_summing_score(folds, n_harmonics: int, *, device=None):
    """Harmonic-sum score of folds ``(..., 2, nbins)``
    (``harmonic_summing_score_func``), float64."""
    device = device or (folds.device if isinstance(folds, torch.Tensor) else "cuda")
    x, host = _to_device(folds, device)
    nb = x.shape[-1]
    flat = x.reshape(-1, 2, nb).contiguous()
    chi, isf = _tables(x.device)
    out = torch.empty(flat.shape[0], dtype=torch.float64, device=x.device)
    _lib.check(_lib.load().loki_harmonic_sum(
        _lib.ptr(flat), flat.shape[0], nb, int(n_harmonics), _lib.ptr(chi), chi.shape[0],
        chi.shape[1], CHI_SQ_RES, CHI_SQ_MAX, _lib.ptr(isf), isf.numel() - 1, MINUS_LOGSF_RES,
        MAX_MINUS_LOGSF, _lib.ptr(out), _lib.stream_ptr(torch.cuda.current_stream(x.device))))
    out = out.reshape(x.shape[:-2])
    return out.cpu().numpy() if host else out

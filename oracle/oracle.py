"""Build and call the C oracle (``loki_oracle.c``) through ctypes.

Test infrastructure only: the checker for the GPU kernels and the timed CPU
baseline. Compiled with ``-O2 -fopenmp -ffp-contract=off`` so that gcc keeps
numpy's rounding (no fused multiply-add) on both x86_64 and aarch64.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "loki_oracle.c"
SOURCES = (SRC, HERE / "prune_oracle.c")
LIB = HERE / "libloki_oracle.so"
CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-std=c11"]

_lib: C.CDLL | None = None
_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int
_D = C.c_double


def build(force: bool = False) -> Path:
    newest = max(s.stat().st_mtime for s in SOURCES)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = str(LIB) + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", *CFLAGS, *map(str, SOURCES), "-o", tmp, "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.oracle_max_threads.restype = C.c_int
        lib.oracle_brutefold.argtypes = [_P, _P, _I64, _P, _I64, _I64, _I32, _D, _D, _P, _I32]
        lib.oracle_ffa_resolve.restype = C.c_double
        lib.oracle_ffa_resolve.argtypes = [_P, _I32, _P, _P, _I32, _I32, _D, _I32, _P]
        lib.oracle_ffa_plan.argtypes = [_I32, _I32, _I32, _D, _P, _P, _P, _P, _P, _P, _P, _P,
                                        _I32]
        lib.oracle_ffa_level.argtypes = [_P, _I64, _I32, _I32, _I32, _D, _P, _P, _P, _P, _P,
                                         _I32]
        lib.oracle_boxcar_snr.argtypes = [_P, _I64, _I32, _P, _I32, _D, _P, _I32]
        lib.oracle_snr_score_batch.argtypes = [_P, _I64, _I32, _P, _I32, _P, _I32]
        lib.oracle_fold_norm.argtypes = [_P, _I64, _I32, _P]
        _lib = lib
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def max_threads() -> int:
    return int(load().oracle_max_threads())


def brutefold(ts_e, ts_v, freqs, segment_len, nbins, tsamp, t_ref=0.0, nthreads=0):
    ts_e = np.ascontiguousarray(ts_e, np.float32)
    ts_v = np.ascontiguousarray(ts_v, np.float32)
    freqs = np.ascontiguousarray(freqs, np.float64)
    nseg = -(-len(ts_e) // segment_len)
    out = np.empty((nseg, len(freqs), 2, nbins), np.float32)
    load().oracle_brutefold(_p(ts_e), _p(ts_v), len(ts_e), _p(freqs), len(freqs), segment_len,
                            nbins, tsamp, t_ref, _p(out), nthreads)
    return out


class _LevelArgs:
    def __init__(self, cfg, level):
        self.n = cfg.nparams
        cur = cfg.get_param_arr(cfg.get_dparams(level))
        self.params = [np.ascontiguousarray(p, np.float64) for p in cur]
        self.ptrs = (C.c_void_p * self.n)(*[p.ctypes.data for p in self.params])
        self.counts_cur = np.array([len(p) for p in cur], np.int64)
        self.counts_prev = np.asarray(cfg.get_param_grid_count(level - 1), np.int64)
        self.limits = np.ascontiguousarray(cfg.param_limits, np.float64)


def ffa_plan(cfg, level, nthreads=0):
    a = _LevelArgs(cfg, level)
    q = int(np.prod(a.counts_cur))
    it = np.empty(q, np.int64)
    ih = np.empty(q, np.int64)
    pt = np.empty(q, np.float64)
    ph = np.empty(q, np.float64)
    load().oracle_ffa_plan(a.n, cfg.nbins, level, cfg.tseg_brute, _p(a.counts_cur),
                           _p(a.counts_prev), _p(a.limits), C.cast(a.ptrs, C.c_void_p),
                           _p(it), _p(pt), _p(ih), _p(ph), nthreads)
    return it, pt, ih, ph


def ffa_level(cfg, level, fold_in, nthreads=0):
    a = _LevelArgs(cfg, level)
    fold_in = np.ascontiguousarray(fold_in, np.float32)
    nseg_in = fold_in.shape[0]
    out = np.empty((nseg_in // 2, *a.counts_cur.tolist(), 2, cfg.nbins), np.float32)
    load().oracle_ffa_level(_p(fold_in), nseg_in, a.n, cfg.nbins, level, cfg.tseg_brute,
                            _p(a.counts_cur), _p(a.counts_prev), _p(a.limits),
                            C.cast(a.ptrs, C.c_void_p), _p(out), nthreads)
    return out


def ffa_initialize(ts_e, ts_v, cfg, nthreads=0):
    freqs = cfg.get_param_arr(cfg.get_dparams(0))[-1]
    t_ref = 0.0 if cfg.nparams == 1 else cfg.bseg_brute * cfg.tsamp / 2
    fold = brutefold(ts_e, ts_v, freqs, cfg.bseg_brute, cfg.nbins, cfg.tsamp, t_ref, nthreads)
    return fold.reshape(fold.shape[0], *([1] * (cfg.nparams - 1)), fold.shape[1], 2, cfg.nbins)


def ffa_execute(ts_e, ts_v, cfg, nthreads=0, keep_levels=False):
    fold = ffa_initialize(ts_e, ts_v, cfg, nthreads)
    levels = [fold]
    for lvl in range(1, cfg.niters_ffa + 1):
        fold = ffa_level(cfg, lvl, fold, nthreads)
        if keep_levels:
            levels.append(fold)
    return levels if keep_levels else fold


def boxcar_snr(prof, widths, stdnoise=1.0, nthreads=0):
    prof = np.ascontiguousarray(prof, np.float32)
    nb = prof.shape[-1]
    flat = prof.reshape(-1, nb)
    widths = np.ascontiguousarray(widths, np.int64)
    out = np.empty((flat.shape[0], len(widths)), np.float32)
    load().oracle_boxcar_snr(_p(flat), flat.shape[0], nb, _p(widths), len(widths), stdnoise,
                             _p(out), nthreads)
    return out.reshape(*prof.shape[:-1], len(widths))


def snr_score_batch(folds, widths, nthreads=0):
    folds = np.ascontiguousarray(folds, np.float32)
    widths = np.ascontiguousarray(widths, np.int64)
    out = np.empty(folds.shape[0], np.float32)
    load().oracle_snr_score_batch(_p(folds), folds.shape[0], folds.shape[-1], _p(widths),
                                  len(widths), _p(out), nthreads)
    return out


def fold_norm(folds):
    folds = np.ascontiguousarray(folds, np.float32)
    nb = folds.shape[-1]
    flat = folds.reshape(-1, 2, nb)
    out = np.empty((flat.shape[0], nb), np.float32)
    load().oracle_fold_norm(_p(flat), flat.shape[0], nb, _p(out))
    return out.reshape(*folds.shape[:-2], nb)


def ffa_trials(ts_e, ts_v, cfg, flat_idx, level=None, seg=0, nthreads=0, f64=False):
    """Fold ``(ntrials, 2, nbins)`` of chosen parameter sets at ``level``
    (default: the final level), segment ``seg``, by single-trial recursion.
    ``f64`` holds and sums every profile in float64 (the FP64 reference)."""
    lib = load()
    if not hasattr(lib, "_trials_bound"):
        for fn in (lib.oracle_ffa_trials, lib.oracle_ffa_trials_f64):
            fn.argtypes = [_P, _P, _I64, _D, _I64, _I32, _I32, _P, _P, _P, _I32,
                           _I64, _P, _I64, _P, _I32]
        lib._trials_bound = True
    level = cfg.niters_ffa if level is None else level
    n = cfg.nparams
    ts_e = np.ascontiguousarray(ts_e, np.float32)
    ts_v = np.ascontiguousarray(ts_v, np.float32)
    grids = [cfg.get_param_arr(cfg.get_dparams(lv)) for lv in range(level + 1)]
    arrs = [np.ascontiguousarray(p, np.float64) for g in grids for p in g]
    ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    counts = np.ascontiguousarray([[len(p) for p in g] for g in grids], np.int64)
    limits = np.ascontiguousarray(cfg.param_limits, np.float64)
    flat_idx = np.ascontiguousarray(flat_idx, np.int64)
    out = np.empty((len(flat_idx), 2, cfg.nbins), np.float64 if f64 else np.float32)
    fn = lib.oracle_ffa_trials_f64 if f64 else lib.oracle_ffa_trials
    fn(_p(ts_e), _p(ts_v), len(ts_e), cfg.tsamp, cfg.bseg_brute, n, cfg.nbins, _p(limits),
       _p(counts), C.cast(ptrs, C.c_void_p), level, seg, _p(flat_idx), len(flat_idx), _p(out),
       nthreads)
    return out


def boxcar_snr_f64(folds, widths, stdnoise=1.0):
    """Boxcar S/N ``(n, nwidths)`` of ``(n, 2, nbins)`` folds with every step in
    float64 (detection/scoring.py:42-71 circular prefix, 99-140 S/N)."""
    folds = np.asarray(folds, np.float64)
    nb = folds.shape[-1]
    widths = np.asarray(widths, np.int64)
    norm = folds[:, 0, :] / np.sqrt(folds[:, 1, :])
    pre = np.cumsum(norm, axis=1)
    total = pre[:, -1:]
    wmax = int(widths.max())
    ext = np.arange(nb + wmax)
    pre_ext = pre[:, ext % nb] + (ext // nb)[None, :] * total
    out = np.empty((len(folds), len(widths)))
    for k, w in enumerate(widths):
        size_w = nb - w
        height = np.sqrt(size_w / (nb * w))
        b = w * height / size_w
        dmax = (pre_ext[:, w:w + nb] - pre_ext[:, :nb]).max(axis=1)
        out[:, k] = ((height + b) * dmax - b * total[:, 0]) / stdnoise
    return out

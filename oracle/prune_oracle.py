"""CPU oracle of the Taylor enumerate-prune run (``prune_oracle.c``).

Test infrastructure only: the checker for the GPU pruning path in tests/ and
the CPU leg of bench.py's pruning measurement. It drives one run the way the
reference's ``Pruning.execute`` does (``prune.py:468-693``): seed from the
reference segment of the FFA fold (``core/taylor.py:14-65``), one
``oracle_prune_level`` per added segment in MiddleOutScheme order, then the
final ascend (``dynamic/dyn_poly_taylor.py:587-628``). The per-level Taylor
matrices and grid-step factors are restated here from the reference's numpy
expressions (``utils/transforms.py:41-45``, ``utils/psr_utils.py:59-95,
227-248``).
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np

from oracle.oracle import _p, load

C_VAL = 299792458.0
MAXP = 5
_M6 = (C.c_double * (MAXP + 1)) * (MAXP + 1)
TILING = {"aggressive": 0, "quadrature": 1, "conservative": 2}


class OPruneLevel(C.Structure):
    _fields_ = [
        ("poly_order", C.c_int), ("nbins", C.c_int), ("nparams_ffa", C.c_int),
        ("moving", C.c_int), ("tiling", C.c_int), ("branch_max", C.c_int),
        ("eta", C.c_double),
        ("dparams_f", C.c_double * MAXP), ("factors", C.c_double * MAXP),
        ("tm_add", _M6), ("tm_init", _M6), ("tm_next", _M6),
        ("dt_phase", C.c_double),
        ("n_accel", C.c_int64), ("n_freq", C.c_int64),
        ("accel_min", C.c_double), ("accel_max", C.c_double),
        ("freq_min", C.c_double), ("freq_max", C.c_double),
    ]


def _fact(k):
    from math import factorial

    k = np.asarray(k)
    return np.vectorize(lambda x: float(factorial(int(x))))(k).astype(np.float64)


def _taylor(dt: float, n: int) -> np.ndarray:
    powers = np.tril(np.arange(n)[:, np.newaxis] - np.arange(n))
    return dt**powers / _fact(powers) * np.tril(np.ones_like(powers))


def _step_f(n: int, tobs: float, nbins: int, eta: float) -> np.ndarray:
    k = np.arange(n)
    d = (eta / nbins) * _fact(k + 1) / tobs ** (k + 1)
    return (2**k * d)[::-1]


def _shift_factors(n: int, tobs: float, nbins: int) -> np.ndarray:
    k = np.arange(n - 1, -1, -1)
    return (tobs - 0) ** (k + 1) * nbins / _fact(k + 1) / 2**k


def _set(dst, m: np.ndarray) -> None:
    for i in range(MAXP + 1):
        for j in range(MAXP + 1):
            dst[i][j] = float(m[i, j]) if i < m.shape[0] and j < m.shape[1] else 0.0


def _bind(lib):
    if getattr(lib, "_prune_bound", False):
        return
    P, I64, I32, D = C.c_void_p, C.c_int64, C.c_int, C.c_double
    lib.oracle_prune_level.restype = I64
    lib.oracle_prune_level.argtypes = [C.POINTER(OPruneLevel), P, P, I64, P, P, I32, D, I64,
                                       I64, P, P, P, P, P, P, I32]
    lib.oracle_prune_ascend.argtypes = [C.POINTER(OPruneLevel), P, P, P, P, I64, I32, P, P,
                                        P, P, I32, I32]
    lib._prune_bound = True


class PruneRun:
    """One enumerate-prune run on the CPU over an FFA fold (numpy)."""

    def __init__(self, cfg, fold: np.ndarray, param_arr, dparams, thresholds, *,
                 max_sugg: int = 2**17, batch_size: int = 1024, moving: bool = True,
                 nthreads: int = 0) -> None:
        from pyloki_gb300.scheme import MiddleOutScheme

        self.cfg = cfg
        self.fold = np.ascontiguousarray(fold, np.float32)
        self.param_arr = param_arr
        self.dparams = np.asarray(dparams, np.float64)
        self.thresholds = np.asarray(thresholds, np.float64)
        self.max_sugg = max_sugg
        self.batch_size = batch_size
        self.moving = moving
        self.nthreads = nthreads
        self.P = cfg.prune_poly_order
        self.widths = np.ascontiguousarray(cfg.score_widths, np.int64)
        self.nseg = self.fold.shape[0]
        self.counts = np.array([len(p) for p in param_arr], np.int64)
        self._scheme_cls = MiddleOutScheme
        self.lib = load()
        _bind(self.lib)

    def _level(self, level: int) -> OPruneLevel:
        cfg, sc, P = self.cfg, self.scheme, self.P
        c_init = sc.get_coord(0)
        c_cur = sc.get_current_coord(level, self.moving)
        c_next = sc.get_coord(level)
        c_add = sc.get_segment_coord(level)
        d = OPruneLevel()
        d.poly_order, d.nbins, d.nparams_ffa = P, cfg.nbins, cfg.nparams
        d.moving = int(self.moving)
        d.tiling = TILING[cfg.tiling_strategy]
        d.branch_max = cfg.branch_max
        d.eta = cfg.eta
        tobs = c_cur[1]
        sf, fa = _step_f(P, tobs, cfg.nbins, cfg.eta), _shift_factors(P, tobs, cfg.nbins)
        for j in range(P):
            d.dparams_f[j] = float(sf[j])
            d.factors[j] = float(fa[j])
        if self.moving:
            _set(d.tm_add, _taylor(c_add[0] - c_cur[0], P + 1))
            _set(d.tm_init, _taylor(c_init[0] - c_cur[0], P + 1))
            _set(d.tm_next, _taylor(c_next[0] - c_cur[0], P + 1))
        else:
            _set(d.tm_add, _taylor(c_add[0] - c_init[0], P + 1))
        d.dt_phase = c_add[0] - c_init[0]
        lim = cfg.param_limits
        d.n_accel, d.n_freq = int(self.counts[-2]), int(self.counts[-1])
        d.accel_min, d.accel_max = float(lim[-2][0]), float(lim[-2][1])
        d.freq_min, d.freq_max = float(lim[-1][0]), float(lim[-1][1])
        return d

    def seed(self, ref_seg: int) -> None:
        from oracle.oracle import snr_score_batch

        P, nb = self.P, self.cfg.nbins
        self.scheme = self._scheme_cls(self.nseg, ref_seg, self.cfg.tseg_ffa, 1)
        mesh = np.meshgrid(*self.param_arr, indexing="ij")
        cart = np.stack([m.ravel() for m in mesh], axis=1)
        n = cart.shape[0]
        f0 = cart[:, -1]
        leaves = np.zeros((n, P + 2, 2), np.float64)
        leaves[:, : P - 1, 0] = cart[:, :-1]
        leaves[:, : P - 1, 1] = self.dparams[:-1]
        leaves[:, -3, 1] = self.dparams[-1] * (C_VAL / f0)
        leaves[:, -1, 0] = f0
        self.leaves = leaves
        self.folds = np.ascontiguousarray(self.fold[self.scheme.ref_idx].reshape(n, 2, nb))
        self.scores = snr_score_batch(self.folds, self.widths, self.nthreads)
        self.scores_ep = self.scores.copy()
        self.backtracks = np.zeros((n, P + 2), np.int32)
        self.level = 0
        self.stats: list[tuple[int, int, int, int]] = []
        self.smm: list[tuple[float, float]] = []
        self.n_leaves_total = 0

    def step(self) -> bool:
        """One level; False once the tree is empty or every segment is added."""
        if self.level >= self.nseg - 1 or len(self.scores) == 0:
            return False
        self.level += 1
        lvl = self.level
        P, nb, cap = self.P, self.cfg.nbins, self.max_sugg
        d = self._level(lvl)
        seg = np.ascontiguousarray(self.fold[self.scheme.get_segment_idx(lvl)])
        lout = np.empty((cap, P + 2, 2), np.float64)
        fout = np.empty((cap, 2, nb), np.float32)
        sout = np.empty(cap, np.float32)
        bout = np.empty((cap, P + 2), np.int32)
        stats = np.zeros(2, np.int64)
        smm = np.zeros(2, np.float64)
        n_par = len(self.scores)
        n = self.lib.oracle_prune_level(
            C.byref(d), _p(self.leaves), _p(self.folds), n_par, _p(seg), _p(self.widths),
            len(self.widths), float(self.thresholds[lvl - 1]), cap, self.batch_size,
            _p(lout), _p(fout), _p(sout), _p(bout), _p(stats), _p(smm), self.nthreads)
        if n == -1:
            msg = "Invalid input: increase branch_max."
            raise ValueError(msg)
        if n < 0:
            msg = "unsupported pruning configuration"
            raise ValueError(msg)
        self.leaves = np.ascontiguousarray(lout[:n])
        self.folds = np.ascontiguousarray(fout[:n])
        self.scores = sout[:n].copy()
        self.scores_ep = self.scores.copy()
        self.backtracks = bout[:n].copy()
        self.stats.append((n_par, int(stats[0]), int(stats[1]), int(n)))
        self.smm.append((float(smm[0]), float(smm[1])))
        self.n_leaves_total += int(stats[0])
        return n > 0

    def ascend(self) -> None:
        n = len(self.scores)
        if n == 0:
            return
        sc, P = self.scheme, self.P
        coord_end = sc.get_previous_coord(self.level + 1, self.moving)
        seg_idx, seg_coords = sc.get_segment_coords_so_far(self.level)
        nseg = len(seg_idx)
        tm = np.zeros((nseg, MAXP + 1, MAXP + 1), np.float64)
        dts = np.zeros(nseg, np.float64)
        for s in range(nseg):
            dt = seg_coords[s, 0] - coord_end[0]
            tm[s, : P + 1, : P + 1] = _taylor(dt, P + 1)
            dts[s] = dt
        segs = [np.ascontiguousarray(self.fold[i]) for i in seg_idx]
        ptrs = (C.c_void_p * nseg)(*[s.ctypes.data for s in segs])
        d = self._level(self.level)
        self.lib.oracle_prune_ascend(
            C.byref(d), _p(self.leaves), _p(self.folds), _p(self.scores), _p(self.scores_ep),
            n, nseg, _p(tm), _p(dts), C.cast(ptrs, C.c_void_p), _p(self.widths),
            len(self.widths), self.nthreads)

    def run(self, ref_seg: int, *, max_levels: int | None = None) -> float:
        """Seed, prune every level (or ``max_levels``), ascend; returns seconds."""
        t0 = time.perf_counter()
        self.seed(ref_seg)
        todo = self.nseg - 1 if max_levels is None else max_levels
        for _ in range(todo):
            if not self.step():
                break
        if max_levels is None:
            self.ascend()
        return time.perf_counter() - t0

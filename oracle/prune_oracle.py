"""CPU oracle of the Taylor, Chebyshev and circular-orbit enumerate-prune runs
(``prune_oracle.c``).

Test infrastructure only: the checker for the GPU pruning path in tests/ and
the CPU leg of bench.py's pruning measurement. It drives one run the way the
reference's ``Pruning.execute`` does (``prune.py:468-693``): seed from the
reference segment of the FFA fold (``core/taylor.py:14-65``), one
``oracle_prune_level`` per added segment in MiddleOutScheme order, then the
final ascend (``dynamic/dyn_poly_taylor.py:587-628``). The per-level Taylor
matrices and grid-step factors are restated here from the reference's numpy
expressions (``utils/transforms.py:41-45``, ``utils/psr_utils.py:59-95,
227-248``). With ``basis="chebyshev"`` the seed is ``poly_chebyshev_seed``
(``core/chebyshev.py:14-72``) and the per-level Chebyshev matrices are
restated from ``utils/maths.py:400-570`` (connection coefficients S and R,
the domain-change matrix C) in the reference's order of evaluation. A
Taylor tree of order 5 is the circular-orbit tree (``PruneCircTaylorDPFuncts``,
the reference's dispatch key ``prune.py:373-381``): Taylor seed and matrices,
plus the classification, validation and closed-form orbit constants of
``core/circular.py`` per level.
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
        ("basis", C.c_int),
        ("cm_prev", _M6), ("cm_add", _M6), ("cm_init", _M6), ("cm_next", _M6),
        ("r_mat", _M6), ("k_fact", C.c_double * (MAXP + 1)),
        ("k_tspow", C.c_double * (MAXP + 1)),
        ("sig_prop", C.c_double), ("sig_val", C.c_double), ("omega_max_sq", C.c_double),
        ("x_mass_const", C.c_double), ("dt_add", C.c_double), ("dt_init", C.c_double),
        ("dt_next", C.c_double),
    ]


# Chebyshev connection coefficients (utils/maths.py:37-52, 400-475) --------------
def _nbinom(n: int, k: int) -> float:
    from math import factorial

    if k < 0 or k > n:
        return 0.0
    if k in (0, n):
        return 1.0
    k = min(k, n - k)
    return float(factorial(n)) // (float(factorial(k)) * float(factorial(n - k)))


def _conn_s(k: int, m: int) -> float:
    """S_{k,m}: x^k in Chebyshev polynomials T_m."""
    if k < 0 or m < 0 or m > k or (k - m) % 2:
        return 0.0
    half = (k - m) // 2
    return 2.0 ** (1 - k - (1 if m == 0 else 0)) * _nbinom(k, half)


def _conn_r(k: int, m: int) -> float:
    """R_{k,m}: T_k in powers x^m."""
    if k < 0 or m < 0 or m > k or (k - m) % 2:
        return 0.0
    if m == 0 and k % 2 == 0:
        return float((-1) ** (k // 2))
    half, mid = (k - m) // 2, (k + m) // 2
    return ((-1) ** half) * (2.0 ** (m - 1)) * (2.0 * k / (k + m)) * _nbinom(mid, half)


def _coef_c(n: int, k: int, p: float, q: float) -> float:
    """C_{n,k}(p, q): T_n of the old domain in T_k of the new one."""
    if k > n:
        return 0.0
    total = 0.0
    for m in range(k, n + 1):
        inner = 0.0
        for i in range(k, m + 1):
            inner += _nbinom(m, i) * p**i * q ** (m - i) * _conn_s(i, k)
        total += _conn_r(n, m) * inner
    return total


def _cheby_matrix(order: int, tc1: float, ts1: float, tc2: float, ts2: float) -> np.ndarray:
    """poly_chebyshev_transform_matrix(order, tc1, ts1, tc2, ts2, 1): the
    domain change of descending coefficients [a_k .. a_0]."""
    p = ts2 / ts1
    q = (tc2 - tc1) / ts1
    size = order + 1
    c = np.zeros((size, size), np.float64)
    for i in range(size):
        for j in range(size):
            c[i, j] = _coef_c(order - i, order - j, p, q)
    return c


def _conn_matrix(fn, order: int) -> np.ndarray:
    m = np.zeros((order + 1, order + 1), np.float64)
    for k in range(order + 1):
        for j in range(k + 1):
            m[k, j] = fn(k, j)
    return m


def _set_rowprod(dst, a: np.ndarray) -> None:
    """x @ a in the oracle's row-product form (row k = column k of a)."""
    _set(dst, np.ascontiguousarray(a.T))


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
    lib.oracle_rowprod.argtypes = [P, I64, I32, P, P]
    lib._prune_bound = True


def _rowprod(lib, x: np.ndarray, a: np.ndarray) -> np.ndarray:
    """x @ a over the last axis with forward fused multiply-adds."""
    m = a.shape[0]
    mat = np.zeros((MAXP + 1, MAXP + 1), np.float64)
    mat[:m, :m] = a.T
    xs = np.ascontiguousarray(x.reshape(-1, m), np.float64)
    out = np.empty_like(xs)
    lib.oracle_rowprod(_p(xs), xs.shape[0], m, _p(mat), _p(out))
    return out.reshape(x.shape)


class PruneRun:
    """One enumerate-prune run on the CPU over an FFA fold (numpy)."""

    def __init__(self, cfg, fold: np.ndarray, param_arr, dparams, thresholds, *,
                 max_sugg: int = 2**17, batch_size: int = 1024, moving: bool = True,
                 nthreads: int = 0, basis: str = "taylor") -> None:
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
        if basis not in ("taylor", "chebyshev"):
            msg = f"basis must be 'taylor' or 'chebyshev', got {basis!r}"
            raise ValueError(msg)
        self.cheby = basis == "chebyshev"
        self.circ = not self.cheby and self.P == 5
        if self.circ and not cfg.p_orb_min > 0:
            msg = "the circular-orbit tree needs p_orb_min"
            raise ValueError(msg)
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
        if self.cheby:
            # poly_cheb_step_vec / poly_cheb_shift_vec (utils/psr_utils.py:259-278)
            # in the Taylor branch's expressions: (dphi * c) / f0 and
            # |dcur - dnew| * (nbins * (f0 / c))
            sf = np.full(P, cfg.eta / cfg.nbins)
            fa = np.full(P, float(cfg.nbins))
        else:
            sf, fa = _step_f(P, tobs, cfg.nbins, cfg.eta), _shift_factors(P, tobs, cfg.nbins)
        for j in range(P):
            d.dparams_f[j] = float(sf[j])
            d.factors[j] = float(fa[j])
        if self.cheby:
            c_prev = sc.get_previous_coord(level, self.moving)
            d.basis = 1
            _set_rowprod(d.cm_prev, _cheby_matrix(P, c_prev[0], c_prev[1], c_cur[0], c_cur[1]))
            t_from = c_cur[0] if self.moving else c_init[0]
            _set_rowprod(d.cm_add, _cheby_matrix(P, t_from, c_cur[1], c_add[0], c_cur[1]))
            _set_rowprod(d.cm_init, _cheby_matrix(P, c_cur[0], c_cur[1], c_init[0], c_cur[1]))
            _set_rowprod(d.cm_next, _cheby_matrix(P, c_cur[0], c_cur[1], c_next[0], c_next[1]))
            self._set_scale(d, c_cur[1])
        elif self.moving:
            _set(d.tm_add, _taylor(c_add[0] - c_cur[0], P + 1))
            _set(d.tm_init, _taylor(c_init[0] - c_cur[0], P + 1))
            _set(d.tm_next, _taylor(c_next[0] - c_cur[0], P + 1))
        else:
            _set(d.tm_add, _taylor(c_add[0] - c_init[0], P + 1))
        if self.circ:  # core/circular.py:83-125, 444-706 and their constants
            d.basis = 2
            d.sig_prop = cfg.propagator_significance
            d.sig_val = cfg.validation_significance
            d.omega_max_sq = (2 * np.pi / cfg.p_orb_min) ** 2
            d.x_mass_const = cfg.x_mass_const
            if self.moving:
                d.dt_add = c_add[0] - c_cur[0]
                d.dt_init = c_init[0] - c_cur[0]
                d.dt_next = c_next[0] - c_cur[0]
            else:
                d.dt_add = c_add[0] - c_init[0]
        d.dt_phase = c_add[0] - c_init[0]
        lim = cfg.param_limits
        d.n_accel, d.n_freq = int(self.counts[-2]), int(self.counts[-1])
        d.accel_min, d.accel_max = float(lim[-2][0]), float(lim[-2][1])
        d.freq_min, d.freq_max = float(lim[-1][0]), float(lim[-1][1])
        return d

    def _set_scale(self, d: OPruneLevel, ts: float) -> None:
        """R and the k! / ts^k scaling of cheby_to_taylor at scale ts."""
        k = np.arange(self.P + 1)
        _set_rowprod(d.r_mat, _conn_matrix(_conn_r, self.P))
        fact = _fact(k)
        tsk = np.float64(ts) ** k
        for i in range(MAXP + 1):
            d.k_fact[i] = float(fact[i]) if i <= self.P else 0.0
            d.k_tspow[i] = float(tsk[i]) if i <= self.P else 1.0

    def _cheby_seed(self, cart: np.ndarray) -> np.ndarray:
        """poly_chebyshev_seed (core/chebyshev.py:14-72): the grid leaves in
        Taylor form (velocity error from the frequency step), then
        taylor_to_cheby_full (utils/transforms.py:458-487) at the initial
        segment's scale."""
        P = self.P
        n = cart.shape[0]
        f0 = cart[:, -1]
        taylor = np.zeros((n, P + 1, 2), np.float64)
        taylor[:, :-2, 0] = cart[:, :-1]
        taylor[:, :-2, 1] = self.dparams[:-1]
        taylor[:, -2, 1] = self.dparams[-1] * (C_VAL / f0)
        k = np.arange(P + 1)
        scale = np.float64(self.scheme.get_coord(0)[1]) ** k / _fact(k)
        s_mat = _conn_matrix(_conn_s, P)
        vals = _rowprod(self.lib, np.ascontiguousarray(taylor[:, ::-1, 0]) * scale, s_mat)
        errs = np.sqrt(_rowprod(self.lib, (np.ascontiguousarray(taylor[:, ::-1, 1]) * scale) ** 2,
                                s_mat**2))
        leaves = np.zeros((n, P + 2, 2), np.float64)
        leaves[:, :-1, 0] = vals[:, ::-1]
        leaves[:, :-1, 1] = errs[:, ::-1]
        leaves[:, -1, 0] = f0
        return leaves

    def seed(self, ref_seg: int) -> None:
        from oracle.oracle import snr_score_batch

        P, nb = self.P, self.cfg.nbins
        self.scheme = self._scheme_cls(self.nseg, ref_seg, self.cfg.tseg_ffa, 1)
        mesh = np.meshgrid(*self.param_arr, indexing="ij")
        cart = np.stack([m.ravel() for m in mesh], axis=1)
        n = cart.shape[0]
        f0 = cart[:, -1]
        if self.cheby:
            leaves = self._cheby_seed(cart)
        else:
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
            if self.cheby:  # core/chebyshev.py:254-300: re-centred at each segment
                tm[s, : P + 1, : P + 1] = _cheby_matrix(
                    P, coord_end[0], coord_end[1], seg_coords[s, 0], coord_end[1]).T
            else:
                tm[s, : P + 1, : P + 1] = _taylor(dt, P + 1)
            dts[s] = dt
        segs = [np.ascontiguousarray(self.fold[i]) for i in seg_idx]
        ptrs = (C.c_void_p * nseg)(*[s.ctypes.data for s in segs])
        d = self._level(self.level)
        if self.cheby:
            self._set_scale(d, coord_end[1])
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

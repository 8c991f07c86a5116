"""Enumerate-prune search on the GPU (drop-in for pyloki's ``prune.py``).

``Pruning`` keeps the reference's interface (``prune.py:347-782``): one
``execute_iter`` per added segment runs the level on the device as

    loki_prune_branch   -> child counts and offsets (one host sync: leaf count)
    loki_prune_score    -> resolve + gather + shift-add + score of every leaf
    loki_prune_select   -> survivors in leaf order (one host sync: survivor count)
    loki_prune_select_overflow  (only when more than ``max_sugg`` survive)
    loki_prune_emit     -> transformed survivors = the new tree

and ``prune_dyp_tree`` runs one pass per reference segment. The per-level
constants (Taylor shift matrices, grid-step factors) are computed here with
the reference's numpy expressions (``core/taylor.py``, ``utils/psr_utils.py``,
``utils/transforms.py``) so the kernels reproduce its arithmetic.

Supported plugins, time-domain folds (``use_fourier=False``), moving or fixed
grid, all three tiling strategies: Taylor basis (``PrunePolyTaylorDPFuncts``),
Chebyshev basis (``PrunePolyChebyshevDPFuncts``) and the circular-orbit Taylor
tree of order 5 (``PruneCircTaylorDPFuncts``, its own branch / map / validate
/ score / emit entry points).
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import itertools
import math
from pathlib import Path

import numpy as np
import torch

from pyloki_gb300 import _lib, chebyshev
from pyloki_gb300.config import C_VAL, FLOAT_EPSILON, fact, poly_taylor_step_f
from pyloki_gb300.scheme import MiddleOutScheme, determine_ref_segs_pareto

_TILING = {"aggressive": 0, "quadrature": 1, "conservative": 2}


def taylor_matrix(delta_t: float, n: int) -> np.ndarray:
    """Lower-triangular Taylor shift matrix (``utils/transforms.py:41-45``)."""
    powers = np.tril(np.arange(n)[:, np.newaxis] - np.arange(n))
    return delta_t**powers / fact(powers) * np.tril(np.ones_like(powers))


def taylor_matrices(delta_t: np.ndarray, n: int) -> np.ndarray:
    """``taylor_matrix`` for every entry of ``delta_t`` at once (the same
    element-wise operations), shape ``(len(delta_t), n, n)``."""
    powers = np.tril(np.arange(n)[:, np.newaxis] - np.arange(n))
    dt = np.asarray(delta_t, dtype=np.float64)[:, np.newaxis, np.newaxis]
    return dt**powers / fact(powers) * np.tril(np.ones_like(powers))


def shift_factors(poly_order: int, tobs: float, nbins: int) -> np.ndarray:
    """Bin-shift factors of poly_taylor_shift_d_vec (``utils/psr_utils.py:227-248``)."""
    k = np.arange(poly_order - 1, -1, -1)
    factors = (tobs - 0) ** (k + 1) * nbins / fact(k + 1)
    return factors / 2**k


def _set6(dst, m: np.ndarray) -> None:
    """Write ``m`` (n x n, n <= 6) into a 6 x 6 ctypes matrix, zero-padded."""
    out = np.ctypeslib.as_array(dst)
    out[...] = 0.0
    n = m.shape[0]
    out[:n, :n] = m


@dataclasses.dataclass
class PruneStats:
    """Statistics of one pruning level (``io/cands.py:17-103``)."""

    level: int
    seg_idx: int
    threshold: float
    score_min: float = 0.0
    score_max: float = 0.0
    n_branches: int = 1
    n_leaves: int = 1
    n_leaves_phy: int = 1
    n_leaves_surv: int = 1

    @property
    def lb_leaves(self) -> float:
        return float(np.round(np.log2(self.n_leaves), 2)) if self.n_leaves else 0.0

    @property
    def branch_frac(self) -> float:
        return 0.0 if self.n_branches == 0 else round(self.n_leaves_phy / self.n_branches, 2)

    @property
    def surv_frac(self) -> float:
        return 0.0 if self.n_leaves_phy == 0 else round(self.n_leaves_surv / self.n_leaves_phy, 2)

    def get_summary(self) -> str:
        return (f"Prune level: {self.level:3d}, seg_idx: {self.seg_idx:3d}, "
                f"leaves: {self.lb_leaves:5.2f}, branch_frac: {self.branch_frac:5.2f}, "
                f"score thresh: {self.threshold:5.2f}, max: {self.score_max:5.2f}, "
                f"min: {self.score_min:5.2f}, P(surv): {self.surv_frac:4.2f}\n")


class WorldTree:
    """Survivor buffer on the device (``utils/world_tree.py:24-178``)."""

    def __init__(self, leaves: torch.Tensor, folds: torch.Tensor, scores: torch.Tensor,
                 backtracks: torch.Tensor, scores_ep: torch.Tensor | None = None) -> None:
        self.leaves = leaves
        self.folds = folds
        self.scores = scores
        self.scores_ep = scores.clone() if scores_ep is None else scores_ep
        self.backtracks = backtracks

    @property
    def valid_size(self) -> int:
        return int(self.scores.shape[0])

    @property
    def size(self) -> int:
        return self.valid_size

    @property
    def nparams(self) -> int:
        return int(self.leaves.shape[1]) - 2

    @property
    def size_lb(self) -> float:
        return float(np.log2(self.valid_size)) if self.valid_size else 0.0

    @property
    def score_max(self) -> float:
        return float(self.scores.max().item()) if self.valid_size else 0.0

    @property
    def score_min(self) -> float:
        return float(self.scores.min().item()) if self.valid_size else 0.0

    def best_k_device(self, k: int) -> tuple[torch.Tensor, torch.Tensor]:
        """Top-k leaves and scores by score, descending, left on the device
        (no host synchronisation); ``get_best_k`` is the host version."""
        k_take = min(k, self.valid_size)
        if k_take == 0:
            return self.leaves[:0], self.scores[:0]
        idx = (torch.argmax(self.scores).reshape(1) if k_take == 1
               else torch.topk(self.scores, k_take).indices)
        return self.leaves[idx], self.scores[idx]

    def take(self, idx: torch.Tensor) -> WorldTree:
        """Rows ``idx`` (device int64, ascending) as a new tree."""
        return WorldTree(self.leaves[idx], self.folds[idx], self.scores[idx],
                         self.backtracks[idx], self.scores_ep[idx])

    def get_best_k(self, k: int) -> tuple[np.ndarray, np.ndarray]:
        """Top-k leaves by score, descending (``world_tree.py:441-459``)."""
        leaves_out = np.zeros((k, *self.leaves.shape[1:]), dtype=np.float64)
        scores_out = np.zeros(k, dtype=np.float32)
        k_take = min(k, self.valid_size)
        if k_take == 0:
            return leaves_out, scores_out
        s = self.scores
        idx = torch.argmax(s).reshape(1) if k_take == 1 else torch.topk(s, k_take).indices
        leaves_out[:k_take] = self.leaves[idx].cpu().numpy()
        scores_out[:k_take] = s[idx].cpu().numpy()
        return leaves_out, scores_out


@dataclasses.dataclass
class PruneIntegrationStep:
    """One hop in a survivor's pruning integration path (``prune.py:334-344``)."""

    level: int
    survivor_idx: int
    seg_idx: int
    parent_idx: int
    param_idx: np.ndarray
    phase_shift: int


class _Buffers:
    """Grow-only device buffers reused across levels."""

    def __init__(self, device) -> None:
        self.device = device
        self.bufs: dict[str, torch.Tensor] = {}

    def get(self, name: str, numel: int, dtype) -> torch.Tensor:
        t = self.bufs.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = torch.empty(max(numel, 1) + (numel >> 3), dtype=dtype, device=self.device)
            self.bufs[name] = t
        return t[:numel]


class Pruning:
    """Enumerate-prune run over one FFA fold (``prune.py:347-782``).

    Parameters
    ----------
    dyp : DynamicProgramming
        FFA with its final level materialised (``execute()``).
    threshold_scheme : array
        One score threshold per pruning level.
    max_sugg : int
        Capacity of the survivor buffer; beyond it the reference's overflow
        rule (top-k / median threshold raise) applies exactly.
    batch_size : int
        Parent batch size of the reference's sequential loop; it only matters
        for the overflow rule, which is batch-sequential.
    """

    def __init__(self, dyp, threshold_scheme, max_sugg: int = 2**17, batch_size: int = 1024,
                 poly_basis: str = "taylor", intermediate_k: int = 1, *,
                 use_moving_grid: bool = True, logger=None) -> None:
        cfg = dyp.cfg
        if dyp.fold.ndim > 8:
            msg = "Pruning currently supports initial data till 5 param dimensions."
            raise ValueError(msg)
        key = (cfg.prune_poly_order == 5, poly_basis, cfg.use_fourier)
        if key not in {(True, "taylor", True), (True, "taylor", False),
                       (False, "taylor", True), (False, "taylor", False),
                       (False, "chebyshev", True), (False, "chebyshev", False)}:
            msg = f"Invalid pruning configuration: {key}"
            raise ValueError(msg)
        self.poly_basis = poly_basis
        #: folds are complex (Fourier domain): (n, 2, nbins / 2 + 1) complex64
        self.fourier = bool(cfg.use_fourier)
        #: the circular-orbit Taylor tree (PruneCircTaylorDPFuncts, poly_order 5)
        self.circular = key[0]
        self._dyp = dyp
        self._threshold_scheme = np.asarray(threshold_scheme, dtype=np.float64)
        self._max_sugg = int(max_sugg)
        self._batch_size = int(batch_size)
        self._intermediate_k = intermediate_k
        self._use_moving_grid = use_moving_grid
        self._logger = logger
        self._lib = _lib.load()
        self._device = dyp.device
        self._buf = _Buffers(self._device)
        self._err = torch.zeros(1, dtype=torch.int32, device=self._device)
        self.poly_order = cfg.prune_poly_order
        self.nparams_ffa = cfg.nparams
        if self.nparams_ffa != self.poly_order or self.nparams_ffa < 2:
            # poly_taylor_seed copies the FFA grid rows into the Taylor rows
            # (core/taylor.py:56-63), which needs one FFA parameter per order.
            msg = (f"the Taylor pruning plugin needs prune_poly_order == FFA parameters "
                   f"(got {self.poly_order} and {self.nparams_ffa})")
            raise ValueError(msg)
        self.spec = _lib.score_spec(cfg.score_widths, cfg.nbins, 1.0, mode=1)
        self.param_grid_count_init = np.asarray(dyp.param_grid_count, np.int64)
        #: kernels launched by this object
        self.launches = 0
        #: if a list, every level appends (start, end) CUDA events recorded on
        #: the launch stream around its loki_prune_score call
        self.score_events: list | None = None
        #: optional ``hook(pruning, tree, level) -> mask | None`` called with the
        #: parents of each Taylor level before branching; a returned device
        #: uint8 mask restricts the level to the parents it marks (their
        #: children still face the exact threshold; backtracks keep the tree's
        #: parent indices). None keeps every parent: the plain algorithm.
        self.parent_hook = None
        #: parents the hook left out, summed over the run
        self.parents_skipped = 0
        #: first child capacity of ``run_device`` (None: max(2^20, 8 max_sugg));
        #: a run that needs more grows it and runs again
        self.device_child_cap: int | None = None

    # ---- reference properties -----------------------------------------------
    @property
    def dyp(self):
        return self._dyp

    @property
    def threshold_scheme(self) -> np.ndarray:
        return self._threshold_scheme

    @property
    def max_sugg(self) -> int:
        return self._max_sugg

    @property
    def batch_size(self) -> int:
        return self._batch_size

    @property
    def intermediate_k(self) -> int:
        return self._intermediate_k

    @property
    def use_moving_grid(self) -> bool:
        return self._use_moving_grid

    @property
    def prune_level(self) -> int:
        return self._prune_level

    @property
    def prune_complete(self) -> bool:
        return self._prune_complete

    @property
    def scheme(self) -> MiddleOutScheme:
        return self._scheme

    @property
    def world_tree(self) -> WorldTree:
        return self._world_tree

    @property
    def pstats(self) -> list[PruneStats]:
        return self._pstats

    @property
    def backtrack_hist(self) -> list[torch.Tensor]:
        return self._backtrack_hist

    @property
    def best_intermediate_arr(self) -> np.ndarray:
        self._flush_best()
        return self._best_intermediate_arr

    def _flush_best(self) -> None:
        """Copy the per-level best leaves recorded on the device to the host
        array (one synchronisation for the whole run)."""
        if self._pending_best:
            bl = self._best_leaves.cpu().numpy()
            bs = self._best_scores.cpu().numpy()
        for row, leaves, scores in self._pending_best:
            slot = self._best_intermediate_arr[row]
            slot["param_sets"][:] = 0
            slot["scores"][:] = 0
            if leaves is None:  # written by loki_prune_best into the run's arrays
                slot["param_sets"][0] = bl[row]
                slot["scores"][0] = bs[row]
                continue
            k = int(scores.shape[0])
            if k:
                slot["param_sets"][:k] = leaves.cpu().numpy()
                slot["scores"][:k] = scores.cpu().numpy()
        self._pending_best = []

    def _record_best(self, level: int, tree: WorldTree) -> None:
        if self.intermediate_k == 1 and tree.valid_size:  # one native launch
            row = int(np.prod(tree.leaves.shape[1:]))
            # rows level - 1 of the run's (levels, row) float64 and (levels,)
            # float32 arrays, addressed directly
            leaf_ptr = self._best_leaves.data_ptr() + (level - 1) * row * 8
            score_ptr = self._best_scores.data_ptr() + (level - 1) * 4
            _lib.check(self._lib.loki_prune_best(
                tree.scores.data_ptr(), tree.valid_size, tree.leaves.data_ptr(), row,
                leaf_ptr, score_ptr, self._stream()))
            self._pending_best.append((level - 1, None, None))
            return
        leaves, scores = tree.best_k_device(self.intermediate_k)
        self._pending_best.append((level - 1, leaves, scores))

    def _stream(self) -> int:
        """The run's stream: the current stream when ``initialize`` ran."""
        ptr = self.__dict__.get("_stream_ptr")
        return ptr if ptr is not None else _lib.stream_ptr(
            torch.cuda.current_stream(self._device))

    def _fold_segment(self, seg: int) -> torch.Tensor:
        f = self.dyp.fold[seg]
        return f.contiguous() if not f.is_contiguous() else f

    # ---- seed (core/taylor.py:14-65, dyn_poly_taylor.py:405-423) -------------
    def _seed(self, fold_segment: torch.Tensor) -> WorldTree:
        cfg = self.dyp.cfg
        P = self.poly_order
        param_arr = self.dyp.param_arr
        dparams = np.asarray(self.dyp.dparams_actual, np.float64)
        mesh = np.meshgrid(*param_arr, indexing="ij")
        cart = np.stack([m.ravel() for m in mesh], axis=1)
        n = cart.shape[0]
        f0 = cart[:, -1]
        df = np.broadcast_to(dparams[-1], (n,))
        leaves = np.zeros((n, P + 2, 2), dtype=np.float64)
        leaves[:, : P - 1, 0] = cart[:, :-1]
        leaves[:, : P - 1, 1] = dparams[:-1]
        leaves[:, -3, 0] = 0
        leaves[:, -3, 1] = df * (C_VAL / f0)
        leaves[:, -2, 0] = 0
        leaves[:, -1, 0] = f0
        leaves[:, -1, 1] = 0
        if self.poly_basis == "chebyshev":  # core/chebyshev.py:14-70
            leaves = chebyshev.seed_leaves(param_arr, dparams, P, self.scheme.get_coord(0)[1])
        from pyloki_gb300.scoring import snr_score_batch

        if self.fourier:  # scored through the irfft (detection/scoring.py:285-292)
            folds = fold_segment.reshape(n, 2, cfg.nbins // 2 + 1).contiguous()
            norm = torch.empty((n, cfg.nbins), dtype=torch.float32, device=self._device)
            _lib.check(self._lib.loki_fold_norm_complex(_lib.ptr(folds), n, cfg.nbins,
                                                        _lib.ptr(norm), self._stream()))
            scores = torch.empty(n, dtype=torch.float32, device=self._device)
            _lib.check(self._lib.loki_boxcar_snr(_lib.ptr(norm), n, cfg.nbins, self.spec,
                                                 _lib.ptr(scores), self._stream()))
        else:
            folds = fold_segment.reshape(n, 2, cfg.nbins).contiguous()
            scores = snr_score_batch(folds, cfg.score_widths)
        bt = torch.zeros((n, P + 2), dtype=torch.int32, device=self._device)
        return WorldTree(torch.from_numpy(leaves).to(self._device), folds, scores, bt)

    def initialize(self, ref_seg: int, log_file: Path | None = None) -> None:
        self._stream_ptr = None
        self._stream_ptr = self._stream()
        self._scheme = MiddleOutScheme(self.dyp.nsegments, ref_seg, self.dyp.tseg, 1)
        self._prune_complete = False
        self._prune_level = 0
        self._world_tree = self._seed(self._fold_segment(self.scheme.ref_idx))
        self._backtrack_hist: list[torch.Tensor] = []
        self._pending_best: list = []
        nlev = max(self.dyp.nsegments - 1, 1)
        self._best_leaves = torch.zeros((nlev, self.poly_order + 2, 2), dtype=torch.float64,
                                        device=self._device)
        self._best_scores = torch.zeros(nlev, dtype=torch.float32, device=self._device)
        self._slots: list = [None, None]
        self._slot_next = 0
        self._work_desc = None
        self._child_cap = max(1 << 20, 64 * self.max_sugg)
        self._ovf_cap = 0
        self._host_words = torch.zeros(4, dtype=torch.int64, pin_memory=True)
        self._pin_n = torch.empty(1, dtype=torch.int64, pin_memory=True)
        self._pin_mm = torch.empty(2, dtype=torch.float32, pin_memory=True)
        self._pin_err = torch.empty(1, dtype=torch.int32, pin_memory=True)
        self._best_intermediate_arr = np.zeros(
            (self.dyp.nsegments - 1, self.intermediate_k),
            dtype=np.dtype([("param_sets", np.float64, (self.poly_order + 2, 2)),
                            ("scores", np.float32)]))
        wt = self._world_tree
        st = PruneStats(level=0, seg_idx=self.scheme.get_segment_idx(0), threshold=0,
                        score_min=wt.score_min, score_max=wt.score_max,
                        n_branches=wt.size, n_leaves=wt.size, n_leaves_phy=wt.size,
                        n_leaves_surv=wt.size)
        self._pstats = [st]
        self._timers: list[np.ndarray] = []
        if log_file is not None:
            with Path(log_file).open("a") as f:
                f.write(st.get_summary())

    # ---- per-level constants ---------------------------------------------------
    def level_desc(self, level: int) -> _lib.LokiPruneLevel:
        """Constants of one level; they depend only on the reference segment
        and the level, so repeated runs from the same segment reuse them. For
        the Taylor basis every level of the segment is built at once
        (``_level_descs_taylor``)."""
        cache = self.__dict__.setdefault("_desc_cache", {})
        if self.poly_basis == "taylor":
            akey = ("taylor_all", self.scheme.ref_idx, self.use_moving_grid)
            if akey not in cache:
                cache[akey] = self._level_descs_taylor(max(self.dyp.nsegments - 1, 1))
            return cache[akey][level - 1]
        key = (self.scheme.ref_idx, level)
        if key not in cache:
            cache[key] = self._level_desc(level)
        return cache[key]

    def _level_descs_taylor(self, nlev: int):
        """``_level_desc`` for levels 1..nlev of the Taylor basis (plain or
        circular-orbit tree) in one vectorised pass (the same element-wise
        operations, so the same values), as a ctypes array of descriptors."""
        cfg = self.dyp.cfg
        sc = self.scheme
        moving = self.use_moving_grid
        P = self.poly_order
        levels = range(1, nlev + 1)
        c_init = sc.get_coord(0)
        cur = np.array([sc.get_current_coord(L, moving) for L in levels], dtype=np.float64)
        nxt = np.array([sc.get_coord(L) for L in levels], dtype=np.float64)
        add = np.array([sc.get_segment_coord(L) for L in levels], dtype=np.float64)
        arr = (_lib.LokiPruneLevel * nlev)()
        v = np.ctypeslib.as_array(arr)
        v["poly_order"] = P
        v["nbins"] = cfg.nbins
        v["nparams_ffa"] = self.nparams_ffa
        v["moving"] = 1 if moving else 0
        v["tiling"] = _TILING[cfg.tiling_strategy]
        v["branch_max"] = cfg.branch_max
        v["eta_m"] = cfg.eta - FLOAT_EPSILON
        tobs = cur[:, 1]
        # poly_taylor_step_f (t_ref 0, Chebyshev-scaled), times c
        k = np.arange(P)
        step = cfg.eta / cfg.nbins * fact(k + 1) / (tobs[:, None] - 0) ** (k + 1)
        step = (2**k * step)[:, ::-1] * C_VAL
        # shift_factors
        kk = np.arange(P - 1, -1, -1)
        fac = (tobs[:, None] - 0) ** (kk + 1) * cfg.nbins / fact(kk + 1) / 2**kk
        v["dfc"][:, :P] = step
        v["fac"][:, :P] = fac
        n = P + 1
        if moving:
            v["tm_a"][:, :n, :n] = taylor_matrices(add[:, 0] - cur[:, 0], n)
            v["tm_i"][:, :n, :n] = taylor_matrices(c_init[0] - cur[:, 0], n)
            tn = taylor_matrices(nxt[:, 0] - cur[:, 0], n)
            v["tm_n"][:, :n, :n] = tn
            v["tm_e"][:, :n, :n] = tn**2 if cfg.tiling_strategy == "quadrature" else np.abs(tn)
        else:
            v["tm_a"][:, :n, :n] = taylor_matrices(add[:, 0] - c_init[0], n)
        v["dt_phase"] = add[:, 0] - c_init[0]
        if self.circular:  # dynamic/dyn_circular_taylor.py:341-385, config.py:475-481
            v["basis"] = 2
            v["circ_sig_prop"] = float(cfg.propagator_significance)
            v["circ_sig_valid"] = float(cfg.validation_significance)
            v["circ_omega_max_sq"] = float((2 * np.pi / cfg.p_orb_min) ** 2)
            v["circ_x_mass"] = float(cfg.x_mass_const)
            if moving:
                v["circ_dt_add"] = add[:, 0] - cur[:, 0]
                v["circ_dt_init"] = c_init[0] - cur[:, 0]
                v["circ_dt_next"] = nxt[:, 0] - cur[:, 0]
            else:
                v["circ_dt_add"] = add[:, 0] - c_init[0]
        counts = self.param_grid_count_init
        lim = cfg.param_limits
        v["n_accel"], v["n_freq"] = int(counts[-2]), int(counts[-1])
        a_min, a_max = lim[-2]
        f_min, f_max = lim[-1]
        v["accel_min"] = float(a_min)
        v["accel_inv"] = float(counts[-2] / (a_max - a_min)) if a_max > a_min else 0.0
        v["freq_min"] = float(f_min)
        v["freq_inv"] = float(counts[-1] / (f_max - f_min)) if f_max > f_min else 0.0
        return arr

    def _level_desc(self, level: int) -> _lib.LokiPruneLevel:
        cfg = self.dyp.cfg
        sc = self.scheme
        moving = self.use_moving_grid
        P = self.poly_order
        coord_init = sc.get_coord(0)
        coord_cur = sc.get_current_coord(level, moving)
        coord_next = sc.get_coord(level)
        coord_add = sc.get_segment_coord(level)
        d = _lib.LokiPruneLevel()
        d.poly_order = P
        d.nbins = cfg.nbins
        d.nparams_ffa = self.nparams_ffa
        d.moving = 1 if moving else 0
        d.tiling = _TILING[cfg.tiling_strategy]
        d.branch_max = cfg.branch_max
        d.eta_m = cfg.eta - FLOAT_EPSILON
        tobs = coord_cur[1]
        dfc = (poly_taylor_step_f(P, tobs, cfg.nbins, cfg.eta, 0)[np.newaxis, :] * C_VAL)[0]
        fac = shift_factors(P, tobs, cfg.nbins)
        for j in range(P):
            d.dfc[j] = float(dfc[j])
            d.fac[j] = float(fac[j])
        if moving:
            _set6(d.tm_a, taylor_matrix(coord_add[0] - coord_cur[0], P + 1))
            _set6(d.tm_i, taylor_matrix(coord_init[0] - coord_cur[0], P + 1))
            tn = taylor_matrix(coord_next[0] - coord_cur[0], P + 1)
            _set6(d.tm_n, tn)
            _set6(d.tm_e, tn**2 if cfg.tiling_strategy == "quadrature" else np.abs(tn))
        else:
            _set6(d.tm_a, taylor_matrix(coord_add[0] - coord_init[0], P + 1))
        d.dt_phase = coord_add[0] - coord_init[0]
        if self.poly_basis == "chebyshev":
            self._cheby_level(d, level, coord_init, coord_cur, coord_next, coord_add)
        if self.circular:  # dynamic/dyn_circular_taylor.py:341-385, config.py:475-481
            d.basis = 2
            d.circ_sig_prop = float(cfg.propagator_significance)
            d.circ_sig_valid = float(cfg.validation_significance)
            d.circ_omega_max_sq = float((2 * np.pi / cfg.p_orb_min) ** 2)
            d.circ_x_mass = float(cfg.x_mass_const)
            if moving:
                d.circ_dt_add = coord_add[0] - coord_cur[0]
                d.circ_dt_init = coord_init[0] - coord_cur[0]
                d.circ_dt_next = coord_next[0] - coord_cur[0]
            else:
                d.circ_dt_add = coord_add[0] - coord_init[0]
        counts = self.param_grid_count_init
        lim = cfg.param_limits
        d.n_accel, d.n_freq = int(counts[-2]), int(counts[-1])
        a_min, a_max = lim[-2]
        f_min, f_max = lim[-1]
        d.accel_min = float(a_min)
        d.accel_inv = float(counts[-2] / (a_max - a_min)) if a_max > a_min else 0.0
        d.freq_min = float(f_min)
        d.freq_inv = float(counts[-1] / (f_max - f_min)) if f_max > f_min else 0.0
        return d

    def _cheby_scale(self, d: _lib.LokiPruneLevel, scale: float) -> None:
        """cheby_to_taylor constants for the domain scale (transforms.py:556-583)."""
        P = self.poly_order
        _set6(d.tm_r, chebyshev.conn_matrix_r(P).T)
        k = np.arange(P + 1, dtype=np.int64)
        cf, tk = fact(k), scale**k
        for i in range(P + 1):
            d.cfact[i] = float(cf[i])
            d.ctsk[i] = float(tk[i])

    def _cheby_level(self, d: _lib.LokiPruneLevel, level: int, coord_init, coord_cur,
                     coord_next, coord_add) -> None:
        """Chebyshev constants of one level (core/chebyshev.py:72-320,
        utils/psr_utils.py:258-278, utils/transforms.py:650-738)."""
        cfg = self.dyp.cfg
        P = self.poly_order
        moving = self.use_moving_grid
        tiling = cfg.tiling_strategy
        d.basis = 1
        dphi = cfg.eta / cfg.nbins
        for j in range(P):
            d.dfc[j] = float((np.zeros(P, np.float64) + dphi)[j] * C_VAL)
            d.fac[j] = float(cfg.nbins)

        def err_matrix(c: np.ndarray) -> np.ndarray:
            return (c**2 if tiling == "quadrature" else np.abs(c)).T

        coord_prev = self.scheme.get_previous_coord(level, moving)
        cb = chebyshev.transform_matrix(P, coord_prev[0], coord_prev[1], coord_cur[0],
                                        coord_cur[1])
        _set6(d.tm_b, cb.T)
        _set6(d.tm_be, err_matrix(cb))
        t0_cur, s_cur = coord_cur
        if moving:
            _set6(d.tm_a, chebyshev.transform_matrix(P, t0_cur, s_cur, coord_add[0], s_cur).T)
            _set6(d.tm_i, chebyshev.transform_matrix(P, t0_cur, s_cur, coord_init[0], s_cur).T)
            cn = chebyshev.transform_matrix(P, t0_cur, s_cur, coord_next[0], coord_next[1])
            _set6(d.tm_n, cn.T)
            _set6(d.tm_e, err_matrix(cn))
        else:  # coord_cur is the fixed-grid coordinate (t0_init, scale)
            _set6(d.tm_a, chebyshev.transform_matrix(P, coord_init[0], s_cur, coord_add[0],
                                                     s_cur).T)
        self._cheby_scale(d, s_cur)

    # ---- one level (prune.py:615-669) ------------------------------------------
    def execute_iter(self, log_file: Path | None = None) -> None:
        if self.prune_complete:
            return
        if self.circular:
            self._execute_iter_circ(log_file)
            return
        if not self.fourier:
            self._execute_iter_native(log_file)
            return
        self._prune_level += 1
        level = self._prune_level
        lib = self._lib
        stream = self._stream()
        seg_idx = self.scheme.get_segment_idx(level)
        fold_segment = self._fold_segment(seg_idx)
        threshold = float(self.threshold_scheme[level - 1])
        d = self.level_desc(level)
        tree = self._world_tree
        mask = self.parent_hook(self, tree, level) if self.parent_hook is not None else None
        n_par = tree.valid_size
        n_expand = n_par
        P = self.poly_order
        offsets = self._buf.get("offsets", n_par + 1, torch.int64)
        info = self._buf.get("info", n_par * _lib.BRANCH_INFO_BYTES, torch.uint8)
        sb = int(lib.loki_scan_scratch_bytes(n_par + 1))
        scan = self._buf.get("scan", sb, torch.uint8)
        if mask is None:
            _lib.check(lib.loki_prune_branch(d, _lib.ptr(tree.leaves), n_par, _lib.ptr(info),
                                             _lib.ptr(offsets), _lib.ptr(scan), sb,
                                             _lib.ptr(self._err), stream))
        else:
            _lib.check(lib.loki_prune_branch_masked(
                d, _lib.ptr(tree.leaves), n_par, _lib.ptr(mask), _lib.ptr(info),
                _lib.ptr(offsets), _lib.ptr(scan), sb, _lib.ptr(self._err), stream))
            n_expand = int(mask.sum().item())
            self.parents_skipped += n_par - n_expand
        # child count and the error word in one wait
        self._pin_n.copy_(offsets[n_par:n_par + 1], non_blocking=True)
        self._pin_err.copy_(self._err, non_blocking=True)
        torch.cuda.current_stream(self._device).synchronize()
        n_child = int(self._pin_n[0])
        if int(self._pin_err[0]):
            _lib.check_dev_err(self._err)
        scores = self._buf.get("cscores", n_child, torch.float32)
        cidx = self._buf.get("cidx", 2 * n_child, torch.int32)
        cphase = self._buf.get("cphase", n_child, torch.float64)
        minmax = self._buf.get("minmax", 2, torch.float32)
        if self.score_events is not None:
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(torch.cuda.current_stream(self._device))
        score_fn = lib.loki_prune_score_complex if self.fourier else lib.loki_prune_score
        _lib.check(score_fn(d, _lib.ptr(tree.leaves), _lib.ptr(tree.folds), n_par,
                                        _lib.ptr(info), _lib.ptr(offsets), n_child,
                                        _lib.ptr(fold_segment), self.spec, _lib.ptr(scores),
                                        _lib.ptr(cidx), _lib.ptr(cphase), _lib.ptr(minmax),
                                        _lib.ptr(self._err), stream))
        if self.score_events is not None:
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record(torch.cuda.current_stream(self._device))
            self.score_events.append((n_child, e0, e1))
        ssb = int(lib.loki_scan_scratch_bytes(n_child)) + 8 * (n_child + 1)
        sscan = self._buf.get("sscan", ssb, torch.uint8)
        surv = self._buf.get("surv", max(n_child, 1), torch.int64)
        n_surv_d = self._buf.get("nsurv", 1, torch.int64)
        _lib.check(lib.loki_prune_select(_lib.ptr(scores), n_child, threshold, _lib.ptr(surv),
                                         _lib.ptr(n_surv_d), _lib.ptr(sscan), ssb, stream))
        # survivor count and score min/max in one transfer and one wait
        self._pin_n.copy_(n_surv_d, non_blocking=True)
        if n_child:
            self._pin_mm.copy_(minmax[:2], non_blocking=True)
        torch.cuda.current_stream(self._device).synchronize()
        n_surv = int(self._pin_n[0])
        mm = self._pin_mm.numpy().copy() if n_child else np.zeros(2, np.float32)
        self.launches += 9
        if n_surv > self.max_sugg:
            n_surv = self._select_overflow(scores, offsets, n_par, n_child, threshold, surv,
                                           n_surv_d)
        nb = self.dyp.cfg.nbins
        dev = self._device
        fold_shape = (n_surv, 2, nb // 2 + 1) if self.fourier else (n_surv, 2, nb)
        new = WorldTree(torch.empty((n_surv, P + 2, 2), dtype=torch.float64, device=dev),
                        torch.empty(fold_shape, dtype=tree.folds.dtype, device=dev),
                        torch.empty(n_surv, dtype=torch.float32, device=dev),
                        torch.empty((n_surv, P + 2), dtype=torch.int32, device=dev),
                        torch.empty(n_surv, dtype=torch.float32, device=dev))
        emit_fn = lib.loki_prune_emit_complex if self.fourier else lib.loki_prune_emit
        _lib.check(emit_fn(d, _lib.ptr(tree.leaves), _lib.ptr(tree.folds),
                                       _lib.ptr(info), _lib.ptr(offsets), n_par,
                                       _lib.ptr(fold_segment), _lib.ptr(surv), n_surv,
                                       _lib.ptr(scores), _lib.ptr(cidx), _lib.ptr(cphase),
                                       _lib.ptr(new.leaves), _lib.ptr(new.folds),
                                       _lib.ptr(new.scores), _lib.ptr(new.scores_ep),
                                       _lib.ptr(new.backtracks), stream))
        self.launches += 1
        st = PruneStats(level=level, seg_idx=seg_idx, threshold=threshold,
                        score_min=float(mm[0]), score_max=float(mm[1]), n_branches=n_expand,
                        n_leaves=n_child, n_leaves_phy=n_child, n_leaves_surv=n_surv)
        self._pstats.append(st)
        if log_file is not None:
            with Path(log_file).open("a") as f:
                f.write(st.get_summary())
        if n_surv == 0:
            self._prune_complete = True
            self._world_tree = new
            return
        self._record_best(level, new)
        self._backtrack_hist.append(new.backtracks)
        self._world_tree = new

    # ---- native level driver (loki_prune_level) ------------------------------
    def _tree_slot(self, k: int, cap: int) -> dict:
        """Ping-pong output tree buffers (capacity ``cap`` rows)."""
        slots = self._slots
        t = slots[k]
        if t is None or t["cap"] < cap:
            P, nb, dev = self.poly_order, self.dyp.cfg.nbins, self._device
            t = slots[k] = {
                "cap": cap,
                "leaves": torch.empty((cap, P + 2, 2), dtype=torch.float64, device=dev),
                "folds": torch.empty((cap, 2, nb), dtype=torch.float32, device=dev),
                "scores": torch.empty(cap, dtype=torch.float32, device=dev),
                "scores_ep": torch.empty(cap, dtype=torch.float32, device=dev),
                "bt": torch.empty((cap, P + 2), dtype=torch.int32, device=dev)}
        return t

    def _work(self, par_cap: int, child_cap: int, ovf_cap: int) -> _lib.LokiPruneWork:
        """The driver's workspace, grown to at least the given capacities."""
        w = self._work_desc
        if (w is not None and w.par_cap >= par_cap and w.child_cap >= child_cap
                and w.ovf_cap >= ovf_cap):
            return w
        lib, b = self._lib, self._buf
        par_cap = max(par_cap, w.par_cap if w is not None else 0)
        child_cap = max(child_cap, w.child_cap if w is not None else 0)
        ovf_cap = max(ovf_cap, w.ovf_cap if w is not None else 0)
        w = _lib.LokiPruneWork()
        w.par_cap, w.child_cap, w.ovf_cap = par_cap, child_cap, ovf_cap
        w.info = b.get("info", par_cap * _lib.BRANCH_INFO_BYTES, torch.uint8).data_ptr()
        w.offsets = b.get("offsets", par_cap + 1, torch.int64).data_ptr()
        w.scan_bytes = int(lib.loki_scan_scratch_bytes(par_cap + 1))
        w.scan = b.get("scan", w.scan_bytes, torch.uint8).data_ptr()
        w.child_scores = b.get("cscores", child_cap, torch.float32).data_ptr()
        w.child_idx = b.get("cidx", 2 * child_cap, torch.int32).data_ptr()
        w.child_phase = b.get("cphase", child_cap, torch.float64).data_ptr()
        w.surv = b.get("surv", max(child_cap, 1), torch.int64).data_ptr()
        w.sscan_bytes = int(lib.loki_scan_scratch_bytes(child_cap)) + 8 * (child_cap + 1)
        w.sscan = b.get("sscan", w.sscan_bytes, torch.uint8).data_ptr()
        w.n_surv = b.get("nsurv", 1, torch.int64).data_ptr()
        w.minmax = b.get("minmax", 2, torch.float32).data_ptr()
        w.ovf_ids = b.get("ovf_ids", ovf_cap, torch.int64).data_ptr()
        w.ovf_keys = b.get("ovf_keys", ovf_cap, torch.float32).data_ptr()
        w.ovf_thr = b.get("ovf_thr", 1, torch.float64).data_ptr()
        w.host_words = self._host_words.data_ptr()
        self._work_desc = w
        return w

    def _execute_iter_native(self, log_file: Path | None = None) -> None:
        self._prune_level += 1
        level = self._prune_level
        seg_idx = self.scheme.get_segment_idx(level)
        fold_segment = self._fold_segment(seg_idx)
        threshold = float(self.threshold_scheme[level - 1])
        d = self.level_desc(level)
        tree = self._world_tree
        mask = self.parent_hook(self, tree, level) if self.parent_hook is not None else None
        n_par = tree.valid_size
        tin = _lib.LokiPruneTree(tree.leaves.data_ptr(), tree.folds.data_ptr(),
                                 tree.scores.data_ptr(), tree.scores_ep.data_ptr(),
                                 tree.backtracks.data_ptr(), n_par, n_par)
        slot = self._tree_slot(self._slot_next, self.max_sugg)
        tout = _lib.LokiPruneTree(slot["leaves"].data_ptr(), slot["folds"].data_ptr(),
                                  slot["scores"].data_ptr(), slot["scores_ep"].data_ptr(),
                                  slot["bt"].data_ptr(), 0, slot["cap"])
        res = _lib.LokiPruneLevelResult()
        w = self._work(max(n_par, self.max_sugg), self._child_cap, self._ovf_cap)
        events = None
        if self.score_events is not None:
            cur = torch.cuda.current_stream(self._device)
            events = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for e in events:  # created on first record; the driver records them again
                e.record(cur)
        while True:
            w.ev_score_begin = events[0].cuda_event if events else None
            w.ev_score_end = events[1].cuda_event if events else None
            rc = self._lib.loki_prune_level(
                d, C.byref(tin), C.byref(tout), C.byref(w), _lib.ptr(fold_segment), self.spec,
                threshold, self.max_sugg, self.batch_size, _lib.ptr(mask), C.byref(res),
                _lib.ptr(self._err), self._stream())
            if rc == _lib.LOKI_ERR_CAPACITY and (res.need_par_cap or res.need_child_cap
                                                 or res.need_ovf_cap):
                self._child_cap = max(self._child_cap, int(res.need_child_cap * 1.25))
                self._ovf_cap = max(self._ovf_cap, int(res.need_ovf_cap * 1.25))
                w = self._work(max(n_par, res.need_par_cap), self._child_cap, self._ovf_cap)
                continue
            _lib.check(rc)
            break
        if res.dev_err:
            _lib.check_dev_err(self._err)
        w.ev_score_begin = w.ev_score_end = None
        if events is not None:
            self.score_events.append((int(res.n_children), events[0], events[1]))
        self.launches += 8 + (1 if res.overflow else 0)
        n_surv = int(res.n_surv)
        n_expand = n_par
        if mask is not None:
            n_expand = int(mask.sum().item())
            self.parents_skipped += n_par - n_expand
        new = WorldTree(slot["leaves"][:n_surv], slot["folds"][:n_surv], slot["scores"][:n_surv],
                        slot["bt"][:n_surv], slot["scores_ep"][:n_surv])
        self._slot_next ^= 1
        n_child = int(res.n_children)
        st = PruneStats(level=level, seg_idx=seg_idx, threshold=threshold,
                        score_min=float(res.score_min) if n_child else 0.0,
                        score_max=float(res.score_max) if n_child else 0.0,
                        n_branches=n_expand, n_leaves=n_child, n_leaves_phy=n_child,
                        n_leaves_surv=n_surv)
        self._pstats.append(st)
        if log_file is not None:
            with Path(log_file).open("a") as f:
                f.write(st.get_summary())
        if n_surv == 0:
            self._prune_complete = True
            self._world_tree = new
            return
        self._record_best(level, new)
        self._backtrack_hist.append(new.backtracks.clone())
        self._world_tree = new

    def _execute_iter_circ(self, log_file: Path | None = None) -> None:
        """One level of the circular-orbit tree (prune.py:165-332 with
        dynamic/dyn_circular_taylor.py): branch with deferred crackle, map the
        batch-ordered children, validate, resolve + score, select, emit."""
        self._prune_level += 1
        level = self._prune_level
        lib = self._lib
        stream = self._stream()
        seg_idx = self.scheme.get_segment_idx(level)
        fold_segment = self._fold_segment(seg_idx)
        threshold = float(self.threshold_scheme[level - 1])
        d = self.level_desc(level)
        tree = self._world_tree
        n_par = tree.valid_size
        P = self.poly_order
        bs = max(1, min(self.batch_size, n_par))
        info = self._buf.get("info", n_par * _lib.BRANCH_INFO_BYTES, torch.uint8)
        keep = self._buf.get("keep", n_par + 1, torch.int64)
        expd = self._buf.get("expd", n_par + 1, torch.int64)
        sb = int(lib.loki_scan_scratch_bytes(n_par + 1))
        scan = self._buf.get("scan", sb, torch.uint8)
        _lib.check(lib.loki_prune_circ_branch(d, _lib.ptr(tree.leaves), n_par, _lib.ptr(info),
                                              _lib.ptr(keep), _lib.ptr(expd), _lib.ptr(scan),
                                              sb, _lib.ptr(self._err), stream))
        n_child = int(keep[n_par].item()) + int(expd[n_par].item())
        _lib.check_dev_err(self._err)
        cmap = self._buf.get("cmap", n_child * _lib.CIRC_CHILD_BYTES, torch.uint8)
        validf = self._buf.get("validf", n_child, torch.float32)
        _lib.check(lib.loki_prune_circ_map(d, _lib.ptr(tree.leaves), n_par, bs, _lib.ptr(info),
                                           _lib.ptr(keep), _lib.ptr(expd), _lib.ptr(cmap),
                                           _lib.ptr(validf), stream))
        vsb = int(lib.loki_scan_scratch_bytes(n_child)) + 8 * (n_child + 1)
        vscan = self._buf.get("vscan", vsb, torch.uint8)
        valid = self._buf.get("valid", max(n_child, 1), torch.int64)
        n_valid_d = self._buf.get("nvalid", 1, torch.int64)
        _lib.check(lib.loki_prune_select(_lib.ptr(validf), n_child, 0.5, _lib.ptr(valid),
                                         _lib.ptr(n_valid_d), _lib.ptr(vscan), vsb, stream))
        n_valid = int(n_valid_d.item())
        scores = self._buf.get("cscores", n_valid, torch.float32)
        cidx = self._buf.get("cidx", 2 * n_valid, torch.int32)
        cphase = self._buf.get("cphase", n_valid, torch.float64)
        ccls = self._buf.get("ccls", n_valid, torch.int8)
        nbatch = (n_par + bs - 1) // bs
        btay = self._buf.get("btay", max(nbatch, 1), torch.int32)
        boff = self._buf.get("boff", n_par + 1, torch.int64)
        minmax = self._buf.get("minmax", 2, torch.float32)
        circ_score = (lib.loki_prune_circ_score_complex if self.fourier
                      else lib.loki_prune_circ_score)
        _lib.check(circ_score(
            d, _lib.ptr(tree.leaves), _lib.ptr(tree.folds), n_par, bs, _lib.ptr(info),
            _lib.ptr(cmap), _lib.ptr(keep), _lib.ptr(expd), _lib.ptr(valid), n_valid,
            _lib.ptr(fold_segment), self.spec, _lib.ptr(scores), _lib.ptr(cidx),
            _lib.ptr(cphase), _lib.ptr(ccls), _lib.ptr(btay), _lib.ptr(boff), _lib.ptr(minmax),
            _lib.ptr(self._err), stream))
        ssb = int(lib.loki_scan_scratch_bytes(n_valid)) + 8 * (n_valid + 1)
        sscan = self._buf.get("sscan", ssb, torch.uint8)
        surv = self._buf.get("surv", max(n_valid, 1), torch.int64)
        n_surv_d = self._buf.get("nsurv", 1, torch.int64)
        _lib.check(lib.loki_prune_select(_lib.ptr(scores), n_valid, threshold, _lib.ptr(surv),
                                         _lib.ptr(n_surv_d), _lib.ptr(sscan), ssb, stream))
        n_surv = int(n_surv_d.item())
        mm = minmax.cpu().numpy() if n_valid else np.zeros(2, np.float32)
        if n_surv > self.max_sugg:
            n_surv = self._select_overflow(scores, boff, n_par, n_valid, threshold, surv,
                                           n_surv_d, batch_size=bs)
        nb = self.dyp.cfg.nbins
        dev = self._device
        fold_shape = (n_surv, 2, nb // 2 + 1) if self.fourier else (n_surv, 2, nb)
        new = WorldTree(torch.empty((n_surv, P + 2, 2), dtype=torch.float64, device=dev),
                        torch.empty(fold_shape, dtype=tree.folds.dtype, device=dev),
                        torch.empty(n_surv, dtype=torch.float32, device=dev),
                        torch.empty((n_surv, P + 2), dtype=torch.int32, device=dev),
                        torch.empty(n_surv, dtype=torch.float32, device=dev))
        circ_emit = lib.loki_prune_circ_emit_complex if self.fourier else lib.loki_prune_circ_emit
        _lib.check(circ_emit(
            d, _lib.ptr(tree.leaves), _lib.ptr(tree.folds), bs, _lib.ptr(info), _lib.ptr(cmap),
            _lib.ptr(valid), _lib.ptr(fold_segment), _lib.ptr(surv), n_surv, _lib.ptr(scores),
            _lib.ptr(cidx), _lib.ptr(cphase), _lib.ptr(ccls), _lib.ptr(btay),
            _lib.ptr(new.leaves), _lib.ptr(new.folds), _lib.ptr(new.scores),
            _lib.ptr(new.scores_ep), _lib.ptr(new.backtracks), stream))
        st = PruneStats(level=level, seg_idx=seg_idx, threshold=threshold,
                        score_min=float(mm[0]), score_max=float(mm[1]), n_branches=n_par,
                        n_leaves=n_child, n_leaves_phy=n_valid, n_leaves_surv=n_surv)
        self._finish_level(st, new, log_file)

    def _finish_level(self, st: PruneStats, new: WorldTree, log_file: Path | None) -> None:
        self._pstats.append(st)
        if log_file is not None:
            with Path(log_file).open("a") as f:
                f.write(st.get_summary())
        if st.n_leaves_surv == 0:
            self._prune_complete = True
            self._world_tree = new
            return
        self._record_best(st.level, new)
        self._backtrack_hist.append(new.backtracks)
        self._world_tree = new

    def _select_overflow(self, scores, offsets, n_par, n_child, threshold, surv, n_surv_d,
                         batch_size: int | None = None) -> int:
        """Exact batch-sequential selection when more than ``max_sugg`` pass."""
        off = offsets.cpu().numpy()
        b = self.batch_size if batch_size is None else batch_size
        starts = np.arange(0, n_par, b)
        ends = np.minimum(starts + b, n_par)
        max_batch = int((off[ends] - off[starts]).max()) if n_par else 0
        n = self.max_sugg + max_batch + 1
        ids = self._buf.get("ovf_ids", n, torch.int64)
        keys = self._buf.get("ovf_keys", n, torch.float32)
        thr_d = self._buf.get("ovf_thr", 1, torch.float64)
        _lib.check(self._lib.loki_prune_select_overflow(
            _lib.ptr(scores), _lib.ptr(offsets), n_par, b, threshold, self.max_sugg,
            _lib.ptr(surv), _lib.ptr(n_surv_d), _lib.ptr(thr_d), _lib.ptr(ids), _lib.ptr(keys),
            n, self._stream()))
        self.launches += 1
        return int(n_surv_d.item())

    def rebind(self, dyp) -> None:
        """Prune the fold of another ``DynamicProgramming`` of the same
        configuration and shape, keeping this object's buffers, level
        constants and captured run graphs (they read the fold through a copy
        made before every device-resident run)."""
        a, b = self.dyp, dyp
        same = (a.fold.shape == b.fold.shape and a.fold.dtype == b.fold.dtype
                and a.device == b.device and a.nsegments == b.nsegments
                and np.array_equal(a.cfg.param_limits, b.cfg.param_limits)
                and all(getattr(a.cfg, k) == getattr(b.cfg, k)
                        for k in ("nsamps", "tsamp", "nbins", "eta", "bseg_brute", "bseg_ffa",
                                  "prune_poly_order", "ducy_max", "wtsp", "use_fourier",
                                  "branch_max", "tiling_strategy")))
        if not same:
            msg = "rebind needs a fold of the same configuration and shape"
            raise ValueError(msg)
        self._dyp = dyp

    # ---- device-resident runs (loki_prune_run) ---------------------------------
    @property
    def device_run_supported(self) -> bool:
        """``run_device`` covers this configuration: the Taylor, Chebyshev and
        circular-orbit trees on time-domain folds, one best leaf per level, no
        parent hook."""
        return not self.fourier and self.intermediate_k == 1 and self.parent_hook is None

    @property
    def block_batch_supported(self) -> bool:
        """``PruneBlockBatch`` covers this configuration: every tree, real or
        complex folds, without a parent hook and with one best leaf per
        level."""
        return self.intermediate_k == 1 and self.parent_hook is None

    def run_device(self, ref_seg: int, *, graph: bool = False, levels: int | None = None) -> None:
        """Every level of one reference segment with the counts kept on the
        device (``loki_prune_run``): the run is enqueued without a host wait
        and read back once at the end (level statistics, survivors, per-level
        best leaves and backtracks), leaving the object as ``initialize`` +
        ``execute_iter`` over all levels (or the first ``levels``) would, before
        the ascend. With
        ``graph=True`` the first run from ``ref_seg`` is captured in a CUDA
        graph that later runs from it replay. The results are those of the
        level-by-level path, kernel for kernel.
        """
        self._device_finish(self._device_enqueue(ref_seg, graph, levels), graph)

    def _device_enqueue(self, ref_seg: int, graph: bool, levels: int | None = None,
                        ascend: bool = False):
        """Enqueue a device-resident run on the current stream (no wait);
        with ``ascend`` the run ends with the ascend over its survivors."""
        if not self.device_run_supported:
            msg = "run_device covers time-domain trees without a parent hook"
            raise ValueError(msg)
        self._stream_ptr = None  # the current stream
        nlev = self.dyp.nsegments - 1 if levels is None else int(levels)
        if not 0 <= nlev <= self.dyp.nsegments - 1:
            msg = f"levels must be in [0, {self.dyp.nsegments - 1}], got {levels}"
            raise ValueError(msg)
        dr = self._device_run_obj(ref_seg, nlev, ascend)
        dr.launch(graph)
        return dr

    def _device_run_obj(self, ref_seg: int, nlev: int, ascend: bool):
        """The cached ``_DeviceRun`` of (reference segment, levels, ascend)."""
        key = (ref_seg, nlev, ascend)
        dr = self.__dict__.setdefault("_device_runs", {}).get(key)
        if dr is None:
            dr = _DeviceRun(self, ref_seg, nlev, ascend=ascend)
            self.__dict__.setdefault("_device_runs", {})[key] = dr
        return dr

    def _device_finish(self, dr, graph: bool) -> None:
        """Read an enqueued run back; repeat it with grown workspaces if it
        outgrew them."""
        while not dr.finish(self):
            key = (dr.ref_seg, dr.nlev, dr.ascend)
            dr = _DeviceRun(self, dr.ref_seg, dr.nlev, grow=dr, ascend=dr.ascend)
            self.__dict__.setdefault("_device_runs", {})[key] = dr
            dr.launch(graph)
        return dr

    # ---- ascend (prune.py:671-693, dyn_poly_taylor.py:587-628) -----------------
    def _ascend_tables(self, level: int):
        """Level descriptor and per-segment tables of the ascend after
        ``level`` (they depend only on the reference segment and the level)."""
        sc = self.scheme
        P = self.poly_order
        coord_end = sc.get_previous_coord(level + 1, self.use_moving_grid)
        seg_idx, seg_coords = sc.get_segment_coords_so_far(level)
        nseg = len(seg_idx)
        cheby = self.poly_basis == "chebyshev"
        dev = self._device
        key = ("ascend", sc.ref_idx, level, self.poly_basis, self.use_moving_grid, str(dev))
        cache = self.__dict__.setdefault("_desc_cache", {})
        if key not in cache:
            dts = seg_coords[:, 0] - coord_end[0]
            tm = np.zeros((nseg, 6, 6), np.float64)
            if cheby:  # core/chebyshev.py:280-320 (shift at the end-domain scale)
                for s in range(nseg):
                    tm[s, : P + 1, : P + 1] = chebyshev.transform_matrix(
                        P, coord_end[0], coord_end[1], seg_coords[s, 0], coord_end[1]).T
            else:
                tm[:, : P + 1, : P + 1] = taylor_matrices(dts, P + 1)
            cache[key] = (torch.from_numpy(tm).to(dev),
                          torch.from_numpy(np.ascontiguousarray(dts, np.float64)).to(dev),
                          torch.from_numpy(seg_idx.astype(np.int32)).to(dev))
        tm_d, dt_d, si_d = cache[key]
        dkey = ("ascend_desc",) + key[1:]
        if dkey not in cache:
            d = _lib.LokiPruneLevel.from_buffer_copy(self._level_desc(level))
            if cheby:
                self._cheby_scale(d, coord_end[1])
            cache[dkey] = d
        return cache[dkey], tm_d, dt_d, si_d, nseg

    def _do_ascend(self) -> None:
        if self.prune_complete or self.world_tree.valid_size == 0:
            return
        d, tm_d, dt_d, si_d, nseg = self._ascend_tables(self.prune_level)
        fold = self.dyp.fold
        stride = int(np.prod(fold.shape[1:]))
        wt = self.world_tree
        ascend_fn = (self._lib.loki_prune_ascend_complex if self.fourier
                     else self._lib.loki_prune_ascend)
        _lib.check(ascend_fn(
            d, _lib.ptr(wt.leaves), _lib.ptr(wt.folds), _lib.ptr(wt.scores),
            _lib.ptr(wt.scores_ep), wt.valid_size, nseg, _lib.ptr(tm_d), _lib.ptr(dt_d),
            _lib.ptr(si_d), _lib.ptr(fold), stride, self.spec, _lib.ptr(self._err),
            self._stream()))
        self.launches += 1

    # ---- report (core/taylor.py:342-360, dyn_poly_cheby.py:824-840) ------------
    def report(self) -> np.ndarray:
        return self._report_host(self.world_tree.leaves.cpu().numpy())

    def _report_host(self, leaves: np.ndarray) -> np.ndarray:
        if self.poly_basis == "chebyshev":
            # The reference's fixed-grid branch computes a shift to the report
            # domain and discards it, so both grids report the leaves as held.
            return chebyshev.report_batch(leaves, self.scheme.get_report_coord(
                self.use_moving_grid))
        return poly_taylor_report_batch(leaves)

    def execute(self, ref_seg: int, ascend_levels: list[int] | None = None,
                outdir: str | Path = "./", log_file: Path | None = None,
                result_file: Path | None = None, task_id: int = 0) -> dict:
        """Full run for one reference segment; returns the run's results.
        Without intermediate ascends the levels run device-resident
        (``run_device``) where the configuration allows, else level by level."""
        asc = frozenset(ascend_levels) if ascend_levels is not None else None
        if asc is None and self.device_run_supported:
            self.run_device(ref_seg)
            if log_file is not None:
                with Path(log_file).open("a") as f:
                    f.writelines(st.get_summary() for st in self.pstats)
        else:
            self.initialize(ref_seg, log_file)
            for _ in range(self.dyp.nsegments - 1):
                self.execute_iter(log_file)
                if asc is not None and self.prune_level in asc:
                    self._do_ascend()
        if asc is None or self.prune_level not in asc:
            self._do_ascend()
        res = {
            "run_name": f"{ref_seg:03d}_{task_id:02d}",
            "scheme": self.scheme.data.copy(),
            "param_sets": self.report(),
            "scores": self.world_tree.scores.cpu().numpy(),
            "scores_ep": self.world_tree.scores_ep.cpu().numpy(),
            "level_stats": self.pstats,
        }
        if result_file is not None:  # prune.py:599-607: the run appended to the file
            from pyloki_gb300.results import PruneResultWriter

            with PruneResultWriter(result_file, mode="a") as writer:
                writer.write_run_results(res["run_name"], res["scheme"], res["param_sets"],
                                         res["scores"], res["scores_ep"], res["level_stats"])
        return res

    def trace_integration_path(self, survivor_idx: int,
                               level: int | None = None) -> list[PruneIntegrationStep]:
        """Walk parent links back to the seed (``prune.py:695-755``)."""
        n_levels = len(self._backtrack_hist)
        if n_levels == 0:
            msg = "No backtrack history; run pruning before tracing a path."
            raise ValueError(msg)
        if level is None:
            level = n_levels
        if not 1 <= level <= n_levels:
            msg = f"level must be in [1, {n_levels}], got {level}"
            raise ValueError(msg)
        steps = []
        lvl, idx = level, survivor_idx
        while lvl >= 1:
            bts = self._backtrack_hist[lvl - 1]
            if idx < 0 or idx >= len(bts):
                msg = f"survivor_idx {idx} out of range [0, {len(bts)}) at level {lvl}"
                raise ValueError(msg)
            bt = bts[idx].cpu().numpy()
            nparams = len(bt) - 2
            steps.append(PruneIntegrationStep(level=lvl, survivor_idx=idx,
                                              seg_idx=self.scheme.get_segment_idx(lvl),
                                              parent_idx=int(bt[0]),
                                              param_idx=bt[1: nparams + 1].copy(),
                                              phase_shift=int(bt[-1])))
            if lvl == 1:
                break
            idx = int(bt[0])
            lvl -= 1
        return steps[::-1]


class _DeviceBuffers:
    """Trees and workspace of device-resident runs on one Pruning object."""

    def __init__(self, prn: Pruning, child_cap: int, bt_rows: int) -> None:
        dev = prn._device
        P, nb, cap = prn.poly_order, prn.dyp.cfg.nbins, prn.max_sugg
        nlev = max(prn.dyp.nsegments - 1, 1)
        lib = prn._lib
        t64, t32, f32, f64, u8 = torch.int64, torch.int32, torch.float32, torch.float64, torch.uint8
        self.child_cap, self.bt_rows = child_cap, bt_rows
        self.host: dict = {}  # pinned readback buffers, grown on demand
        fold_row = ((2, nb // 2 + 1), torch.complex64) if prn.fourier else ((2, nb), f32)
        self.trees = [{"leaves": torch.empty((cap, P + 2, 2), dtype=f64, device=dev),
                       "folds": torch.empty((cap, *fold_row[0]), dtype=fold_row[1],
                                            device=dev),
                       "scores": torch.empty(cap, dtype=f32, device=dev),
                       "scores_ep": torch.empty(cap, dtype=f32, device=dev),
                       "bt": torch.empty((cap, P + 2), dtype=t32, device=dev)} for _ in range(2)]
        scan_bytes = int(lib.loki_scan_scratch_bytes(cap + 1))
        sscan_bytes = int(lib.loki_scan_scratch_bytes(child_cap)) + 8 * (child_cap + 1)
        ovf_cap = cap + child_cap + 1
        self.mem = {
            "info": torch.empty(cap * _lib.BRANCH_INFO_BYTES, dtype=u8, device=dev),
            "offsets": torch.empty(cap + 1, dtype=t64, device=dev),
            "scan": torch.empty(scan_bytes, dtype=u8, device=dev),
            "cscores": torch.empty(child_cap, dtype=f32, device=dev),
            "cidx": torch.empty(2 * child_cap, dtype=t32, device=dev),
            "cphase": torch.empty(child_cap, dtype=f64, device=dev),
            "surv": torch.empty(child_cap, dtype=t64, device=dev),
            "sscan": torch.empty(sscan_bytes, dtype=u8, device=dev),
            "minmax": torch.empty(2, dtype=f32, device=dev),
            "ovf_ids": torch.empty(ovf_cap, dtype=t64, device=dev),
            "ovf_keys": torch.empty(ovf_cap, dtype=f32, device=dev),
            "ovf_thr": torch.empty(1, dtype=f64, device=dev),
            "counts": torch.zeros(8, dtype=t64, device=dev),
            "ovf_flag": torch.zeros(1, dtype=t32, device=dev),
            "stats": torch.zeros(nlev * _lib.PRUNE_STATS_DTYPE.itemsize, dtype=u8, device=dev),
            "best_leaves": torch.zeros((nlev, P + 2, 2), dtype=f64, device=dev),
            "best_scores": torch.zeros(nlev, dtype=f32, device=dev),
            "bt_hist": torch.empty((bt_rows, P + 2), dtype=t32, device=dev),
            # the FFA fold the runs read: a copy made on the stream before each
            # run, so a captured graph serves any fold of the same shape
            "mirror": torch.empty(int(prn.dyp.fold.numel()), dtype=prn.dyp.fold.dtype,
                                  device=dev),
            "seed_scores": torch.empty(cap, dtype=f32, device=dev),
        }
        m = self.mem
        r = _lib.LokiPruneRun()
        for k, t in enumerate(self.trees):
            r.trees[k] = _lib.LokiPruneTree(t["leaves"].data_ptr(), t["folds"].data_ptr(),
                                            t["scores"].data_ptr(), t["scores_ep"].data_ptr(),
                                            t["bt"].data_ptr(), 0, cap)
        w = r.work
        w.info, w.offsets, w.scan = (m["info"].data_ptr(), m["offsets"].data_ptr(),
                                     m["scan"].data_ptr())
        w.scan_bytes, w.par_cap = scan_bytes, cap
        w.child_scores, w.child_idx = m["cscores"].data_ptr(), m["cidx"].data_ptr()
        w.child_phase, w.surv = m["cphase"].data_ptr(), m["surv"].data_ptr()
        w.sscan, w.sscan_bytes, w.child_cap = m["sscan"].data_ptr(), sscan_bytes, child_cap
        w.n_surv, w.minmax = None, m["minmax"].data_ptr()
        w.ovf_ids, w.ovf_keys = m["ovf_ids"].data_ptr(), m["ovf_keys"].data_ptr()
        w.ovf_thr, w.ovf_cap = m["ovf_thr"].data_ptr(), ovf_cap
        r.counts, r.ovf_flag, r.stats = (m["counts"].data_ptr(), m["ovf_flag"].data_ptr(),
                                         m["stats"].data_ptr())
        r.best_leaves, r.best_scores = m["best_leaves"].data_ptr(), m["best_scores"].data_ptr()
        r.bt_hist, r.bt_rows = m["bt_hist"].data_ptr(), bt_rows
        if prn.circular:  # the circular tree's own child bookkeeping
            nbatch = cap // max(1, prn.batch_size) + 1
            m.update({
                "exp_off": torch.empty(cap + 1, dtype=t64, device=dev),
                "cmap": torch.empty(child_cap * _lib.CIRC_CHILD_BYTES, dtype=u8, device=dev),
                "validf": torch.empty(child_cap, dtype=f32, device=dev),
                "valid": torch.empty(child_cap, dtype=t64, device=dev),
                "ccls": torch.empty(child_cap, dtype=torch.int8, device=dev),
                "btay": torch.empty(nbatch, dtype=t32, device=dev),
                "boff": torch.empty(cap + 1, dtype=t64, device=dev)})
            r.exp_off, r.child_map = m["exp_off"].data_ptr(), m["cmap"].data_ptr()
            r.valid_flags, r.valid_ids = m["validf"].data_ptr(), m["valid"].data_ptr()
            r.child_class, r.batch_taylor = m["ccls"].data_ptr(), m["btay"].data_ptr()
            r.batch_offsets = m["boff"].data_ptr()
        self.run = r


class _DeviceRun:
    """One reference segment's device-resident run: level descriptors,
    segment order, thresholds, the seed (copied into the first tree at the
    start of every run) and, once captured, the run's CUDA graph."""

    def __init__(self, prn: Pruning, ref_seg: int, nlev: int,
                 grow: _DeviceRun | None = None, ascend: bool = False) -> None:
        dyp = prn.dyp
        nseg = dyp.nsegments
        self.nlev = nlev
        self.ref_seg = ref_seg
        self.scheme = MiddleOutScheme(nseg, ref_seg, dyp.tseg, 1)
        prn._scheme = self.scheme
        self.seed = prn._seed(prn._fold_segment(ref_seg))
        if self.seed.size > prn.max_sugg:
            msg = "the seed tree is larger than max_sugg"
            raise ValueError(msg)
        cap = prn.max_sugg
        bufs = prn.__dict__.get("_device_bufs")
        child_cap = prn.device_child_cap or max(1 << 20, 8 * cap)
        bt_rows = max(1, min(self.nlev * cap, max(1 << 22, 16 * cap)))
        if grow is not None:
            child_cap = max(child_cap, grow.need_child, bufs.child_cap if bufs else 0)
            bt_rows = max(bt_rows, grow.need_bt, bufs.bt_rows if bufs else 0)
        if (bufs is None or bufs.child_cap < child_cap or bufs.bt_rows < bt_rows
                or bufs.mem["mirror"].numel() < dyp.fold.numel()):
            prn.__dict__.pop("_device_runs", None)  # their graphs hold the old buffers
            bufs = prn._device_bufs = _DeviceBuffers(prn, child_cap, bt_rows)
        self.bufs = bufs
        self.descs = (_lib.LokiPruneLevel * max(self.nlev, 1))()
        for lvl in range(1, self.nlev + 1):
            C.memmove(C.byref(self.descs, (lvl - 1) * C.sizeof(_lib.LokiPruneLevel)),
                      C.byref(prn.level_desc(lvl)), C.sizeof(_lib.LokiPruneLevel))
        self.seg_idx = np.ascontiguousarray(
            [self.scheme.get_segment_idx(lvl) for lvl in range(1, self.nlev + 1)], np.int32)
        self.thresholds = np.ascontiguousarray(prn.threshold_scheme[: self.nlev], np.float64)
        self.ascend = bool(ascend) and self.nlev > 0
        self.asc = prn._ascend_tables(self.nlev) if self.ascend else None
        self.prn = prn
        self.graph = None
        self.need_child = self.need_bt = 0

    def _fold_src(self):
        """The FFA fold the run reads: the run's mirror (a captured graph
        keeps its address across folds) or, for the batched drivers, the
        fold itself."""
        return self.__dict__.get("_direct_fold", self.bufs.mem["mirror"])

    def _seed_enqueue(self) -> None:
        """The seed tree from the fold: leaves from the grid, folds and
        scores from the reference segment's rows (complex rows scored
        through their irfft, as ``Pruning._seed``)."""
        prn, b = self.prn, self.bufs
        t0, seed = b.trees[0], self.seed
        n = seed.size
        nb = prn.dyp.cfg.nbins
        stride = int(np.prod(prn.dyp.fold.shape[1:]))
        src = self._fold_src()
        t0["leaves"][:n].copy_(seed.leaves)
        t0["folds"][:n].copy_(src[self.ref_seg * stride:(self.ref_seg + 1) * stride]
                              .view(n, *t0["folds"].shape[1:]))
        if prn.fourier:
            norm = torch.empty((n, nb), dtype=torch.float32, device=prn._device)
            _lib.check(prn._lib.loki_fold_norm_complex(_lib.ptr(t0["folds"]), n, nb,
                                                       _lib.ptr(norm), prn._stream()))
            _lib.check(prn._lib.loki_boxcar_snr(_lib.ptr(norm), n, nb, prn.spec,
                                                _lib.ptr(t0["scores"]), prn._stream()))
        else:
            _lib.check(prn._lib.loki_snr_score_batch(
                _lib.ptr(t0["folds"]), n, nb, prn.spec, _lib.ptr(t0["scores"]),
                prn._stream()))
        t0["scores_ep"][:n].copy_(t0["scores"][:n])
        b.mem["seed_scores"][:n].copy_(t0["scores"][:n])  # level-0 statistics
        t0["bt"][:n].zero_()
        prn._err.zero_()

    def _ascend_enqueue(self) -> None:
        """The ascend over the last level's survivors (counts[0] after the run)."""
        prn, b = self.prn, self.bufs
        stride = int(np.prod(prn.dyp.fold.shape[1:]))
        d, tm_d, dt_d, si_d, nseg = self.asc
        t = b.trees[self.nlev & 1]
        _lib.check(prn._lib.loki_prune_ascend_dev(
            d, _lib.ptr(t["leaves"]), _lib.ptr(t["folds"]), _lib.ptr(t["scores"]),
            _lib.ptr(t["scores_ep"]), _lib.ptr(b.mem["counts"]), prn.max_sugg, nseg,
            _lib.ptr(tm_d), _lib.ptr(dt_d), _lib.ptr(si_d), _lib.ptr(self._fold_src()), stride,
            prn.spec, _lib.ptr(prn._err), prn._stream()))

    def ascend_job(self) -> _lib.LokiAscendJob:
        """This run's ascend as a job of ``loki_prune_ascend_batch``."""
        prn, b = self.prn, self.bufs
        d, tm_d, dt_d, si_d, _ = self.asc
        t = b.trees[self.nlev & 1]
        j = _lib.LokiAscendJob()
        j.lvl = d
        j.leaves, j.folds = _lib.ptr(t["leaves"]), _lib.ptr(t["folds"])
        j.scores, j.scores_ep = _lib.ptr(t["scores"]), _lib.ptr(t["scores_ep"])
        j.n_dev = _lib.ptr(b.mem["counts"])
        j.tm_seg, j.dt_seg, j.seg_idx = _lib.ptr(tm_d), _lib.ptr(dt_d), _lib.ptr(si_d)
        j.ffa_fold = _lib.ptr(self._fold_src())
        j.seg_stride = int(np.prod(prn.dyp.fold.shape[1:]))
        j.dev_err = _lib.ptr(prn._err)
        return j

    def tree_parts(self, n: int):
        """(device tensor, bytes) of the final tree's first n rows: leaves,
        scores, scores_ep."""
        t = self.bufs.trees[self.nlev & 1]
        P = self.prn.poly_order
        return [(t["leaves"], n * (P + 2) * 2 * 8), (t["scores"], n * 4),
                (t["scores_ep"], n * 4)]

    def job(self) -> _lib.LokiPruneJob:
        """This run as a job of the batched drivers (after the seed)."""
        prn, b = self.prn, self.bufs
        j = _lib.LokiPruneJob()
        j.ffa_fold = _lib.ptr(self._fold_src())
        j.seg_stride = int(np.prod(prn.dyp.fold.shape[1:]))
        j.seed_n = self.seed.size
        j.run = b.run
        j.dev_err = _lib.ptr(prn._err)
        return j

    def prepare_block(self) -> None:
        """The seed, read from the fold itself, for a batched driver."""
        self._direct_fold = self.prn.dyp.fold.reshape(-1)
        self._seed_enqueue()

    def seed_job(self) -> _lib.LokiSeedJob:
        """This run's seed as a job of ``loki_prune_seed_batch``, reading the
        fold itself."""
        prn, b = self.prn, self.bufs
        self._direct_fold = prn.dyp.fold.reshape(-1)
        t0, n = b.trees[0], self.seed.size
        stride = int(np.prod(prn.dyp.fold.shape[1:]))
        j = _lib.LokiSeedJob()
        j.seed_leaves = _lib.ptr(self.seed.leaves)
        j.fold_rows = _lib.ptr(self._direct_fold) + 4 * self.ref_seg * stride
        j.n = n
        j.leaves_out, j.folds_out = _lib.ptr(t0["leaves"]), _lib.ptr(t0["folds"])
        j.scores_out, j.scores_ep_out = _lib.ptr(t0["scores"]), _lib.ptr(t0["scores_ep"])
        j.seed_scores_out = _lib.ptr(b.mem["seed_scores"])
        j.bt_out = _lib.ptr(t0["bt"])
        j.dev_err = _lib.ptr(prn._err)
        return j

    def _enqueue(self) -> None:
        """The run from the fold mirror: the seed, then every level."""
        prn, b = self.prn, self.bufs
        self._seed_enqueue()
        if self.nlev == 0:
            return
        stride = int(np.prod(prn.dyp.fold.shape[1:]))
        _lib.check(prn._lib.loki_prune_run(
            self.descs, self.nlev, _lib.ptr(b.mem["mirror"]), stride, self.seg_idx.ctypes.data,
            self.thresholds.ctypes.data, prn.spec, self.seed.size, prn.max_sugg,
            prn.batch_size, C.byref(b.run), _lib.ptr(prn._err), prn._stream()))
        if self.ascend:
            self._ascend_enqueue()

    def launch(self, graph: bool) -> None:
        self.__dict__.pop("_direct_fold", None)  # the graphs read the mirror
        fold = self.prn.dyp.fold.reshape(-1)
        self.bufs.mem["mirror"][: fold.numel()].copy_(fold)  # outside any graph
        if not graph:
            self._enqueue()
            return
        if self.graph is None:
            self._enqueue()  # uncaptured first run: kernel attributes, lazy loading
            cur = torch.cuda.current_stream(self.prn._device)
            side = torch.cuda.Stream(self.prn._device)
            side.wait_stream(cur)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(side):
                self.prn._stream_ptr = _lib.stream_ptr(side)
                with torch.cuda.graph(g, stream=side):
                    self._enqueue()
            cur.wait_stream(side)
            self.prn._stream_ptr = _lib.stream_ptr(cur)
            self.graph = g
        self.graph.replay()

    def _pinned(self, name: str, numel: int, dtype) -> torch.Tensor:
        """Grow-only pinned host buffer of the run's buffers."""
        b = self.bufs
        t = b.host.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = b.host[name] = torch.empty(max(numel, 1), dtype=dtype, pin_memory=True)
        return t[:numel]

    def copy_stats_async(self) -> None:
        """Enqueue the copies of the level records, error word and seed
        scores to pinned host memory on the current stream."""
        prn, b = self.prn, self.bufs
        nbytes = self.nlev * _lib.PRUNE_STATS_DTYPE.itemsize
        self._h_stats = self._pinned("stats", nbytes, torch.uint8)
        self._h_stats.copy_(b.mem["stats"][:nbytes], non_blocking=True)
        self._h_err = self._pinned("err", 1, torch.int32)
        self._h_err.copy_(prn._err, non_blocking=True)
        self._h_seed = self._pinned("seed", self.seed.size, torch.float32)
        self._h_seed.copy_(b.mem["seed_scores"][: self.seed.size], non_blocking=True)

    def stats_host(self):
        """(level records, error word, last level, survivors of it) from the
        pinned copies (after the stream has been waited on)."""
        stats = self._h_stats.numpy().view(_lib.PRUNE_STATS_DTYPE)
        err = int(self._h_err[0])
        if self.nlev == 0:
            return stats, err, 0, self.seed.size
        n_surv = stats["n_surv"][: self.nlev]
        dead = np.flatnonzero(n_surv == 0)  # the run stops at its first empty level
        last = int(dead[0]) + 1 if dead.size else self.nlev
        return stats, err, last, int(n_surv[last - 1])

    def copy_tree_async(self, n: int) -> None:
        """Enqueue the copies of the final tree's first n rows (leaves, scores,
        scores_ep) to pinned host memory on the current stream."""
        t = self.bufs.trees[self.nlev & 1]
        P = self.prn.poly_order
        self._h_leaves = self._pinned("leaves", n * (P + 2) * 2, torch.float64)
        self._h_leaves.copy_(t["leaves"][:n].reshape(-1), non_blocking=True)
        self._h_scores = self._pinned("scores", n, torch.float32)
        self._h_scores.copy_(t["scores"][:n], non_blocking=True)
        self._h_scores_ep = self._pinned("scores_ep", n, torch.float32)
        self._h_scores_ep.copy_(t["scores_ep"][:n], non_blocking=True)

    def level_stats(self, stats, last: int) -> list[PruneStats]:
        sc, seed = self.scheme, self.seed
        s0 = self._h_seed.numpy()
        out = [PruneStats(level=0, seg_idx=sc.get_segment_idx(0), threshold=0,
                          score_min=float(s0.min()) if seed.size else 0.0,
                          score_max=float(s0.max()) if seed.size else 0.0,
                          n_branches=seed.size, n_leaves=seed.size, n_leaves_phy=seed.size,
                          n_leaves_surv=seed.size)]
        f = stats[:last]
        nch = f["n_children"]
        # positional fields (level, seg_idx, threshold, score_min, score_max,
        # n_branches, n_leaves, n_leaves_phy, n_leaves_surv); a level without
        # children has no score range
        out.extend(itertools.starmap(PruneStats, zip(
            range(1, last + 1), self.seg_idx[:last].tolist(), self.thresholds[:last].tolist(),
            np.where(nch != 0, f["score_min"], 0.0).tolist(),
            np.where(nch != 0, f["score_max"], 0.0).tolist(), f["n_parents"].tolist(),
            nch.tolist(), f["n_valid"].tolist(), f["n_surv"].tolist())))
        return out

    def finish(self, prn: Pruning) -> bool:
        """Read the run back (one wait) and set ``prn``'s state; False when a
        workspace has to grow (``need_*`` set) and the run must be repeated."""
        b = self.bufs
        stats = b.mem["stats"].cpu().numpy().view(_lib.PRUNE_STATS_DTYPE)
        err = int(prn._err.item())
        if err & _lib.LOKI_DEVERR_CAPACITY:
            self.need_child = int(stats["n_children"].max() * 1.25) + 1
            self.need_bt = int(stats["n_surv"].sum() * 1.25) + 1
            prn._err.zero_()
            return False
        if err:
            _lib.check_dev_err(prn._err)
        sc = self.scheme
        prn._scheme = sc
        seed = self.seed
        s0 = b.mem["seed_scores"][: seed.size]
        st0 = PruneStats(level=0, seg_idx=sc.get_segment_idx(0), threshold=0,
                         score_min=float(s0.min()) if seed.size else 0.0,
                         score_max=float(s0.max()) if seed.size else 0.0,
                         n_branches=seed.size, n_leaves=seed.size, n_leaves_phy=seed.size,
                         n_leaves_surv=seed.size)
        pstats = [st0]
        bt_hist = []
        off = 0
        bt = b.mem["bt_hist"]
        last = 0
        for lvl in range(1, self.nlev + 1):
            r = stats[lvl - 1]
            n_child, n_surv = int(r["n_children"]), int(r["n_surv"])
            pstats.append(PruneStats(
                level=lvl, seg_idx=int(self.seg_idx[lvl - 1]),
                threshold=float(self.thresholds[lvl - 1]),
                score_min=float(r["score_min"]) if n_child else 0.0,
                score_max=float(r["score_max"]) if n_child else 0.0,
                n_branches=int(r["n_parents"]), n_leaves=n_child,
                n_leaves_phy=int(r["n_valid"]), n_leaves_surv=n_surv))
            last = lvl
            if n_surv == 0:
                break
            bt_hist.append(bt[off:off + n_surv])
            off += n_surv
        n_final = int(stats[last - 1]["n_surv"]) if last else seed.size
        t = b.trees[last & 1]
        prn._pstats = pstats
        prn._prune_level = last
        prn._prune_complete = n_final == 0
        prn._world_tree = WorldTree(t["leaves"][:n_final], t["folds"][:n_final],
                                    t["scores"][:n_final], t["bt"][:n_final],
                                    t["scores_ep"][:n_final])
        prn._backtrack_hist = bt_hist
        nkeep = len(bt_hist)
        prn._best_leaves = b.mem["best_leaves"]
        prn._best_scores = b.mem["best_scores"]
        prn._pending_best = [(lvl - 1, None, None) for lvl in range(1, nkeep + 1)]
        prn._best_intermediate_arr = np.zeros(
            (prn.dyp.nsegments - 1, prn.intermediate_k),
            dtype=np.dtype([("param_sets", np.float64, (prn.poly_order + 2, 2)),
                            ("scores", np.float32)]))
        prn.launches += 1 + 13 * self.nlev
        return True


def poly_taylor_report_batch(leaves: np.ndarray) -> np.ndarray:
    """Gauge transform of the final leaves (``core/taylor.py:342-360``)."""
    out = leaves.copy()
    vals = leaves[:, :-3, 0]
    sigs = leaves[:, :-3, 1]
    v_final = leaves[:, -3, 0]
    dv_final = leaves[:, -3, 1]
    f0 = leaves[:, -1, 0]
    s = 1 - v_final / C_VAL
    out[:, :-3, 0] = vals / s[:, None]
    out[:, :-3, 1] = np.sqrt((sigs / s[:, None]) ** 2
                             + ((vals / (C_VAL * s[:, None] ** 2)) ** 2) * (dv_final[:, None] ** 2))
    out[:, -3, 0] = f0 * s
    out[:, -3, 1] = f0 * dv_final / C_VAL
    return out


def prune_dyp_tree(dyp, threshold_scheme, n_runs: int | None = None,
                   ref_segs: list[int] | None = None, ascend_levels: list[int] | None = None,
                   max_sugg: int = 2**18, batch_size: int = 1024, outdir: str | Path = "./",
                   file_prefix: str = "test", poly_basis: str = "taylor", *,
                   use_moving_grid: bool = True, n_workers: int = 4,
                   driver: str = "auto") -> str:
    """Prune from several reference segments (``prune.py:824-932``).

    ``driver="auto"`` runs every segment at once on the device
    (``PruneBlockBatch``: one launch per step of a level over all runs)
    when the tree supports device-resident runs and only the final ascend is
    asked for; otherwise, and with ``driver="threads"``, ``n_workers`` runs
    proceed at once, each on its own host thread and CUDA stream
    (``run_many``). Every run is the same computation as on its own.
    Results are written as the reference's HDF5 result file
    (``PruneResultWriter``: file attributes, ``threshold_scheme`` and
    ``runs/<ref:03d>_<task:02d>/{scheme, param_sets, scores_ep, scores,
    level_stats, timer_stats}``), runs in ``ref_segs`` order.
    """
    if driver not in ("auto", "threads"):
        msg = f"driver must be 'auto' or 'threads', got {driver!r}"
        raise ValueError(msg)
    if not isinstance(n_workers, int | np.integer):
        msg = f"n_workers must be an integer, got {type(n_workers)}"
        raise TypeError(msg)
    if n_workers < 1:
        msg = f"n_workers must be greater than 0, got {n_workers}"
        raise ValueError(msg)
    if n_runs is not None:
        if not 1 <= n_runs <= dyp.nsegments:
            msg = f"n_runs must be between 1 and {dyp.nsegments}, got {n_runs}"
            raise ValueError(msg)
        ref_segs = determine_ref_segs_pareto(dyp.nsegments, n_runs)
    elif ref_segs is None:
        msg = "Either n_runs or ref_segs must be provided"
        raise ValueError(msg)
    outdir = Path(outdir)
    outdir.mkdir(parents=True, exist_ok=True)
    filebase = f"{file_prefix}_pruning_nstages_{dyp.nsegments}"
    log_file = outdir / f"{filebase}_log.txt"
    result_file = outdir / f"{filebase}_results.h5"
    if log_file.exists() or result_file.exists():
        msg = f"{log_file} or {result_file} already exists"
        raise FileExistsError(msg)
    log_file.write_text("Pruning log\n")
    kw = {"max_sugg": max_sugg, "batch_size": batch_size, "poly_basis": poly_basis,
          "use_moving_grid": use_moving_grid}
    probe = Pruning(dyp, threshold_scheme, **kw)
    batched = driver == "auto" and ascend_levels is None and probe.block_batch_supported
    if batched:
        res_list = PruneBlockBatch(threshold_scheme, **kw).run([(dyp, r) for r in ref_segs])
        results = dict(zip(ref_segs, res_list, strict=True))
    else:
        results = run_many(dyp, threshold_scheme, ref_segs, n_workers=n_workers,
                           ascend_levels=ascend_levels, **kw)
    from pyloki_gb300.results import PruneResultWriter

    with PruneResultWriter(result_file) as writer:
        writer.write_metadata(dyp.cfg.param_names, dyp.nsegments, max_sugg, threshold_scheme)
        for ref_seg in ref_segs:
            res = results[ref_seg]
            with log_file.open("a") as f:
                f.write(f"Pruning log for ref segment: {ref_seg}\n")
                for st in res["level_stats"]:
                    f.write(st.get_summary())
            writer.write_run_results(res["run_name"], res["scheme"], res["param_sets"],
                                     res["scores"], res["scores_ep"], res["level_stats"])
    return result_file.as_posix()


class PruneBatch:
    """Device-resident runs of many (fold, reference segment) jobs at once
    from one host thread (``loki_prune_run``).

    Job i of a call goes to stream i mod ``n_streams``; every stream keeps
    one ``Pruning`` (rebound to each job's fold of the same configuration),
    its run buffers and, per reference segment, the run's CUDA graph (with
    ``graph``), so repeated calls, over the same or new folds, only copy the
    fold and replay graphs. A round enqueues one run per stream with no host wait, so the
    streams' small per-level kernels overlap on the GPU, then reads the round
    back (one wait per run) and, with ``ascend``, re-folds the survivors over
    all segments. Every run is the same computation as ``Pruning.execute``
    on its own.
    """

    def __init__(self, threshold_scheme, *, n_streams: int = 8, graph: bool = True,
                 **kwargs) -> None:
        if int(n_streams) < 1:
            msg = f"n_streams must be greater than 0, got {n_streams}"
            raise ValueError(msg)
        self.threshold_scheme = threshold_scheme
        self.n_streams = int(n_streams)
        self.graph = graph
        self.kwargs = kwargs
        self._streams: list = []
        self._prns: list[dict] = []  # per stream: {"prn": Pruning}
        self._bufs: list = []

    def _stream(self, k: int, dev):
        while len(self._streams) <= k:
            self._streams.append(torch.cuda.Stream(dev))
            self._prns.append({})
            self._bufs.append(None)
        return self._streams[k]

    def _pruning(self, k: int, dyp) -> Pruning:
        prn = self._prns[k].get("prn")
        if prn is not None and prn.dyp is not dyp:
            try:
                prn.rebind(dyp)
            except ValueError:
                prn = None
        if prn is None:
            prn = self._prns[k]["prn"] = Pruning(dyp, self.threshold_scheme, **self.kwargs)
            if self._bufs[k] is not None:
                prn._device_bufs = self._bufs[k]
        return prn

    def run(self, jobs, *, ascend: bool = True) -> list[dict]:
        """``jobs``: a list of ``(dyp, ref_seg)``; returns ``execute``'s
        dictionaries in job order."""
        jobs = list(jobs)
        if not jobs:
            return []
        dev = jobs[0][0].device
        producer = torch.cuda.current_stream(dev)
        ns = min(self.n_streams, len(jobs))
        out: list[dict] = [{} for _ in jobs]
        for r0 in range(0, len(jobs), ns):
            started = []
            for k, (dyp, ref) in enumerate(jobs[r0:r0 + ns]):
                st = self._stream(k, dev)
                st.wait_stream(producer)
                with torch.cuda.stream(st):
                    prn = self._pruning(k, dyp)
                    dr = prn._device_enqueue(ref, self.graph, ascend=ascend)
                    dr.copy_stats_async()
                started.append((k, prn, dr))
            # one wait per run for its records, then the surviving rows
            ready = []
            for k, prn, dr in started:
                st = self._streams[k]
                st.synchronize()
                stats, err, last, n = dr.stats_host()
                with torch.cuda.stream(st):
                    if err:  # a workspace to grow, or a device error to raise
                        dr = prn._device_finish(dr, self.graph)
                        dr.copy_stats_async()
                        st.synchronize()
                        stats, err, last, n = dr.stats_host()
                    dr.copy_tree_async(n)
                self._bufs[k] = prn._device_bufs
                ready.append((k, prn, dr, stats, last, n))
            P = ready[0][1].poly_order
            for k, prn, dr, stats, last, n in ready:
                self._streams[k].synchronize()
                prn._scheme = dr.scheme
                leaves = dr._h_leaves.numpy().reshape(n, P + 2, 2).copy()
                out[r0 + k] = {
                    "run_name": f"{dr.ref_seg:03d}_00", "scheme": dr.scheme.data.copy(),
                    "param_sets": prn._report_host(leaves),
                    "scores": dr._h_scores.numpy().copy(),
                    "scores_ep": dr._h_scores_ep.numpy().copy(),
                    "level_stats": dr.level_stats(stats, last)}
        for st in self._streams[:ns]:
            producer.wait_stream(st)
        return out


class PruneBlockBatch(PruneBatch):
    """Device-resident runs of many (fold, reference segment) jobs enqueued
    together. ``driver="batch"`` (``loki_prune_run_batch``): every step of a
    level is one launch over all jobs, so the batch pays the launches of one
    run. ``driver="blocks"`` (``loki_prune_run_blocks``): one thread block
    per job walks every level with block barriers between the steps, a
    single launch for the batch.

    Up to ``max_jobs`` jobs go in one launch, each with its own ``Pruning``
    and run buffers (kept across calls, rebound to each job's fold). The
    ascend, the read-back and the results are those of ``PruneBatch``; a job
    that outgrows its workspace is repeated with grown buffers through
    the same driver. Taylor, Chebyshev and circular-orbit trees over real
    folds, and (with the level-synchronous driver) over complex folds; the
    block-per-run driver passes circular-orbit trees to ``PruneBatch``.
    """

    def __init__(self, threshold_scheme, *, max_jobs: int = 152, driver: str = "batch",
                 **kwargs) -> None:
        super().__init__(threshold_scheme, n_streams=1, graph=False, **kwargs)
        if int(max_jobs) < 1:
            msg = f"max_jobs must be greater than 0, got {max_jobs}"
            raise ValueError(msg)
        if driver not in ("batch", "blocks"):
            msg = f"driver must be 'batch' or 'blocks', got {driver!r}"
            raise ValueError(msg)
        self.max_jobs = int(max_jobs)
        self.driver = driver
        self._slots: list = []
        self._scratch = None

    def _enqueue_batch(self, lib, dev, st, n: int, nlev: int, args, shape) -> None:
        """The batch's kernels over the tables just copied: enqueued directly
        the first time a shape is seen, then captured once in a CUDA graph
        and replayed (the tables are read on the device, so a replay runs
        whatever jobs were copied in)."""
        if self.__dict__.get("time_score"):  # measurement: uncaptured, timed score launches
            ms = np.zeros(nlev, np.float32)
            _lib.check(lib.loki_prune_batch_score_times(
                _lib.ptr(self._scratch), n, nlev, *args, shape.ctypes.data, ms.ctypes.data,
                _lib.stream_ptr(st)))
            self.score_ms = ms
            return
        key = (n, nlev, tuple(int(v) for v in shape), args[1], args[2])
        graphs = self.__dict__.setdefault("_graphs", {})
        g = graphs.get(key)
        if g is None and key not in self.__dict__.setdefault("_seen", set()):
            self._seen.add(key)
            _lib.check(lib.loki_prune_batch_enqueue(_lib.ptr(self._scratch), n, nlev, *args,
                                                    shape.ctypes.data, _lib.stream_ptr(st)))
            return
        if g is None:
            side = torch.cuda.Stream(dev)
            side.wait_stream(st)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(side), torch.cuda.graph(g, stream=side):
                _lib.check(lib.loki_prune_batch_enqueue(
                    _lib.ptr(self._scratch), n, nlev, *args, shape.ctypes.data,
                    _lib.stream_ptr(side)))
            st.wait_stream(side)
            graphs[key] = g
        g.replay()

    def _slot(self, k: int, dyp) -> Pruning:
        while len(self._slots) <= k:
            self._slots.append(None)
        prn = self._slots[k]
        if prn is not None and prn.dyp is not dyp:
            try:
                prn.rebind(dyp)
            except ValueError:
                prn = None
        if prn is None:
            prn = self._slots[k] = Pruning(dyp, self.threshold_scheme, **self.kwargs)
        return prn

    def run(self, jobs, *, ascend: bool = True) -> list[dict]:
        jobs = list(jobs)
        if not jobs:
            return []
        first = self._slot(0, jobs[0][0])
        if not first.block_batch_supported:
            msg = ("the batched drivers cover trees without a parent hook and with one best "
                   "leaf per level")
            raise ValueError(msg)
        fourier = first.fourier
        if fourier and self.driver == "blocks":
            msg = "complex (Fourier-domain) trees run with driver='batch'"
            raise ValueError(msg)
        if first.circular and self.driver == "blocks":
            return PruneBatch.run(self, jobs, ascend=ascend)
        dev = jobs[0][0].device
        st = torch.cuda.current_stream(dev)
        out: list[dict] = [{} for _ in jobs]
        lib = _lib.load()
        for w0 in range(0, len(jobs), self.max_jobs):
            wave = jobs[w0:w0 + self.max_jobs]
            runs = []
            for k, (dyp, ref) in enumerate(wave):
                prn = self._slot(k, dyp)
                prn._stream_ptr = None  # the current stream
                runs.append((prn, prn._device_run_obj(ref, dyp.nsegments - 1, ascend)))
            self._run_jobs(lib, dev, st, runs, ascend, fourier)
            # a job that outgrew its workspace is repeated, through the same
            # driver, with grown buffers (the others keep their results)
            todo = list(range(len(runs)))
            for attempt in range(17):  # each round grows the workspaces by at least 1.25x
                grown = []
                for i in todo:
                    prn, dr = runs[i]
                    err = int(dr._h_err[0])
                    if err & _lib.LOKI_DEVERR_CAPACITY:
                        stats = dr._h_stats.numpy().view(_lib.PRUNE_STATS_DTYPE)
                        dr.need_child = int(stats["n_children"].max() * 1.25) + 1
                        dr.need_bt = int(stats["n_surv"].sum() * 1.25) + 1
                        prn._err.zero_()
                        new = _DeviceRun(prn, dr.ref_seg, dr.nlev, grow=dr, ascend=dr.ascend)
                        prn.__dict__.setdefault("_device_runs", {})[
                            (dr.ref_seg, dr.nlev, dr.ascend)] = new
                        runs[i] = (prn, new)
                        grown.append(i)
                    elif err:
                        _lib.check_dev_err(prn._err)
                if not grown:
                    break
                if attempt == 16:
                    msg = "pruning runs still outgrow their workspaces after 16 enlargements"
                    raise RuntimeError(msg)
                self._run_jobs(lib, dev, st, [runs[i] for i in grown], ascend, fourier)
                todo = grown
            ready = []
            for prn, dr in runs:
                stats, _, last, nf = dr.stats_host()
                ready.append((prn, dr, stats, last, nf))
            host = self._read_trees(lib, dev, st, ready)
            P = ready[0][0].poly_order
            for i, (prn, dr, stats, last, nf) in enumerate(ready):
                prn._scheme = dr.scheme
                leaves_b, scores_b, ep_b = host[i]
                leaves = np.frombuffer(leaves_b, np.float64).reshape(nf, P + 2, 2).copy()
                out[w0 + i] = {
                    "run_name": f"{dr.ref_seg:03d}_00", "scheme": dr.scheme.data.copy(),
                    "param_sets": prn._report_host(leaves),
                    "scores": np.frombuffer(scores_b, np.float32).copy(),
                    "scores_ep": np.frombuffer(ep_b, np.float32).copy(),
                    "level_stats": dr.level_stats(stats, last)}
        return out

    def _run_jobs(self, lib, dev, st, runs, ascend: bool, fourier: bool) -> None:
        """Seeds, levels and ascends of ``runs`` (one slot each), then every
        job's level records, error word and seed scores on the host (one
        gather and one copy)."""
        nlev = runs[0][1].nlev
        n = len(runs)
        if not fourier and all(prn.dyp.fold.dtype == torch.float32 for prn, _ in runs):
            sjobs = (_lib.LokiSeedJob * n)()  # every job's seed in one launch
            for i, (prn, dr) in enumerate(runs):
                sjobs[i] = dr.seed_job()
            p0 = runs[0][0]
            sbuf = self._dev_buf("seed", n * C.sizeof(_lib.LokiSeedJob), dev)
            _lib.check(lib.loki_prune_seed_batch(
                sjobs, n, p0.dyp.cfg.nbins, p0.poly_order, p0.spec, _lib.ptr(sbuf),
                sbuf.numel(), _lib.stream_ptr(st)))
        else:  # complex folds, or a fold stored in another type: per-job seeds
            for prn, dr in runs:
                dr.prepare_block()
        if nlev > 0:
            tab = (_lib.LokiPruneJob * n)()
            for i, (prn, dr) in enumerate(runs):
                tab[i] = dr.job()
            lv, seg, thr = self._level_tables(runs, nlev)
            need = int(lib.loki_prune_run_blocks_scratch_bytes(n, nlev))
            if self._scratch is None or self._scratch.numel() < need:
                self._scratch = torch.empty(need, dtype=torch.uint8, device=dev)
                self._graphs = {}  # captured over the old scratch
            p0 = runs[0][0]
            args = (p0.spec, p0.max_sugg, p0.batch_size)
            if self.driver == "blocks":
                _lib.check(lib.loki_prune_run_blocks(
                    tab, n, lv, seg.ctypes.data, thr.ctypes.data, nlev, *args,
                    _lib.ptr(self._scratch), self._scratch.numel(), _lib.stream_ptr(st)))
            else:
                shape = np.zeros(6, np.int64)
                _lib.check(lib.loki_prune_batch_tables(
                    tab, n, lv, seg.ctypes.data, thr.ctypes.data, nlev, *args,
                    int(fourier), _lib.ptr(self._scratch), self._scratch.numel(),
                    shape.ctypes.data, _lib.stream_ptr(st)))
                self._enqueue_batch(lib, dev, st, n, nlev, args, shape)
        if ascend and nlev > 0:  # every job's ascend in one launch
            ajobs = (_lib.LokiAscendJob * n)()
            for i, (prn, dr) in enumerate(runs):
                ajobs[i] = dr.ascend_job()
            p0 = runs[0][0]
            abuf = self._dev_buf("ascend", n * C.sizeof(_lib.LokiAscendJob), dev)
            _lib.check(lib.loki_prune_ascend_batch(
                ajobs, n, runs[0][1].asc[4], p0.spec, p0.max_sugg, int(fourier),
                _lib.ptr(abuf), abuf.numel(), _lib.stream_ptr(st)))
        isz = _lib.PRUNE_STATS_DTYPE.itemsize
        raw = self._gather_read(
            lib, dev, st, [[(dr.bufs.mem["stats"], dr.nlev * isz), (prn._err, 4),
                            (dr.bufs.mem["seed_scores"], dr.seed.size * 4)]
                           for prn, dr in runs], "stats")
        for (prn, dr), (b_st, b_err, b_seed) in zip(runs, raw, strict=True):
            dr._h_stats = torch.from_numpy(np.frombuffer(b_st, np.uint8).copy())
            dr._h_err = torch.from_numpy(np.frombuffer(b_err, np.int32).copy())
            dr._h_seed = torch.from_numpy(np.frombuffer(b_seed, np.float32).copy())

    def _level_tables(self, runs, nlev: int):
        """Level descriptors (in pinned memory, so that their copy to the
        device is one DMA), segment order and thresholds of ``runs``, job
        after job. They depend only on each run's configuration, reference
        segment and levels, so a call over the same runs (new folds or not)
        reuses them."""
        key = tuple((id(prn), dr.ref_seg, dr.nlev, id(dr)) for prn, dr in runs)
        cached = self.__dict__.get("_lv_cache")
        if cached is not None and cached[0] == key:
            return cached[1:4]
        n = len(runs)
        size = C.sizeof(_lib.LokiPruneLevel)
        nbytes = n * nlev * size
        pin = self.__dict__.get("_lv_pin")
        if pin is None or pin.numel() < nbytes:
            pin = self._lv_pin = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        lv = (_lib.LokiPruneLevel * (n * nlev)).from_address(pin.data_ptr())
        seg = np.empty((n, nlev), np.int32)
        thr = np.empty((n, nlev), np.float64)
        for i, (_, dr) in enumerate(runs):
            C.memmove(C.byref(lv, i * nlev * size), dr.descs, nlev * size)
            seg[i] = dr.seg_idx
            thr[i] = dr.thresholds
        self._lv_cache = (key, lv, seg, thr, pin)
        return lv, seg, thr

    def _dev_buf(self, name: str, nbytes: int, dev):
        bufs = self.__dict__.setdefault("_dev_bufs", {})
        t = bufs.get(name)
        if t is None or t.numel() < nbytes:
            t = bufs[name] = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
        return t

    def _read_trees(self, lib, dev, st, ready):
        """Every job's final rows (leaves, scores, scores_ep)."""
        return self._gather_read(lib, dev, st, [dr.tree_parts(nf) for _, dr, _, _, nf in ready],
                                 "trees")

    def _gather_read(self, lib, dev, st, groups, name: str):
        """Device ranges (per job a list of (tensor, bytes)) packed on the
        device by one gather launch and read back with one copy; returns the
        bytes of every range, per job."""
        parts, offs, off = [], [], 0
        for group in groups:
            row = []
            for t, nb in group:
                parts.append((t, nb, off))
                row.append((off, nb))
                off += (nb + 15) // 16 * 16
            offs.append(row)
        packed = self._dev_buf(f"packed_{name}", off, dev)
        pins = self.__dict__.setdefault("_pins", {})
        pin = pins.get(name)
        if pin is None or pin.numel() < off:
            pin = pins[name] = torch.empty(max(off, 256), dtype=torch.uint8, pin_memory=True)
        tab = (_lib.LokiGatherPart * len(parts))()
        for i, (t, nb, o) in enumerate(parts):
            tab[i].src, tab[i].bytes, tab[i].dst_off = _lib.ptr(t), nb, o
        pbuf = self._dev_buf(f"parts_{name}", len(parts) * C.sizeof(_lib.LokiGatherPart), dev)
        _lib.check(lib.loki_gather_parts(tab, len(parts), _lib.ptr(packed), packed.numel(),
                                         _lib.ptr(pbuf), pbuf.numel(), _lib.stream_ptr(st)))
        if off:
            pin[:off].copy_(packed[:off], non_blocking=True)
        st.synchronize()
        raw = pin.numpy()
        return [[raw[o:o + nb].tobytes() for o, nb in row] for row in offs]


def run_batch(jobs, threshold_scheme, *, n_streams: int = 8, graph: bool = True,
              ascend: bool = True, **kwargs) -> list[dict]:
    """``PruneBatch(...).run(jobs)`` once (graphs and buffers are not kept)."""
    return PruneBatch(threshold_scheme, n_streams=n_streams, graph=graph,
                      **kwargs).run(jobs, ascend=ascend)


def run_many(dyp, threshold_scheme, ref_segs, *, n_workers: int = 4,
             ascend_levels: list[int] | None = None, **kwargs) -> dict[int, dict]:
    """``Pruning.execute`` for every reference segment, ``n_workers`` at a
    time on separate host threads and CUDA streams; results by segment."""
    import threading

    ref_segs = list(ref_segs)
    dev = dyp.device
    producer = torch.cuda.current_stream(dev)
    work = list(ref_segs)
    results: dict[int, dict] = {}
    errors: list[BaseException] = []
    lock = threading.Lock()
    streams = [torch.cuda.Stream(dev) for _ in range(max(1, min(n_workers, len(ref_segs))))]

    def worker(stream) -> None:
        try:
            stream.wait_stream(producer)  # the fold is ready before any run reads it
            with torch.cuda.device(dev), torch.cuda.stream(stream):
                prn = Pruning(dyp, threshold_scheme, **kwargs)
                while True:
                    with lock:
                        if not work or errors:
                            return
                        ref = work.pop(0)
                    before = prn.launches
                    res = prn.execute(ref, ascend_levels=ascend_levels)
                    res["launches"] = prn.launches - before
                    with lock:
                        results[ref] = res
        except BaseException as e:  # noqa: BLE001 - re-raised in the caller
            with lock:
                errors.append(e)

    if len(streams) == 1:
        worker(streams[0])
    else:
        threads = [threading.Thread(target=worker, args=(st,)) for st in streams]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    for st in streams:
        producer.wait_stream(st)
    if errors:
        raise errors[0]
    return results


def leaves_per_second(stats: list[PruneStats], seconds: float) -> float:
    """Prune leaves/s: leaves emitted by branch (``n_leaves``) over the run time."""
    return float(sum(s.n_leaves for s in stats[1:])) / seconds if seconds > 0 else math.inf

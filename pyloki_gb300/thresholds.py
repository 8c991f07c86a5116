"""Threshold-scheme design on the GPU (drop-in for pyloki's
``detection/thresholding.py``).

The reference designs the per-level pruning thresholds by Monte Carlo: folded
profiles of pure noise (H0) and of noise plus a template pulse (H1) are grown
stage by stage (``simulate_folds``, ``thresholding.py:46-96``), scored with the
boxcar S/N (``fold_max_scores``, ``484-500``) and cut at a threshold
(``prune_folds``, ``99-135``); survival rates drive a dynamic programme over
(stage, threshold, H1-survival bin) states (``DynamicThresholdScheme``,
``702-1008``), or evaluate a given scheme (``evaluate_scheme``, ``1062-1110``)
or a given set of survival probabilities (``determine_scheme``, ``1010-1059``).

Here every simulation and scoring of a stage runs as one launch over all the
fold sets of the stage (``loki_sim_score_folds``), survivors are compacted
with ``loki_gather_rows``, and only the scores come back to the host, where
the state bookkeeping (a few thousand small records) follows the reference's
rules. The noise comes from a counter-based generator keyed by ``seed``, so a
design is reproducible (the reference draws from an unseeded
``np.random.default_rng()``); results therefore agree with the reference in
distribution, not draw for draw.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Literal

import numpy as np
import torch
from scipy import stats

from pyloki_gb300 import _lib
from pyloki_gb300.config import generate_box_width_trials

state_dtype = np.dtype(
    [("success_h0", np.float32), ("success_h1", np.float32), ("complexity", np.float32),
     ("complexity_cumul", np.float32), ("success_h1_cumul", np.float32),
     ("nbranches", np.float32), ("threshold", np.float32), ("cost", np.float32),
     ("threshold_prev", np.float32), ("success_h1_cumul_prev", np.float32),
     ("is_empty", np.bool_)],
)


def generate_folded_profile(nbins: int = 100, ducy: float = 0.1,
                            center: float = 0.5) -> np.ndarray:
    """Unit-norm Gaussian pulse profile (``simulation/pulse.py:512-523``):
    FWHM-style width from the duty cycle, peak normalised then L2-normalised."""
    phase = np.linspace(0, 1, nbins, endpoint=False)
    sigma = ducy / (2 * np.sqrt(2 * np.log(10)))
    wrapped = np.mod(phase - center + 0.5, 1) - 0.5
    prof = np.exp(-(wrapped**2) / (2 * sigma**2))
    prof = prof / prof.max()
    return prof / np.sqrt(np.sum(prof**2))


def bound_scheme(nstages: int, snr_bound: float) -> np.ndarray:
    """Thresholds with S/N^2 growing linearly to ``snr_bound^2``
    (``detection/schemes.py:29-50``)."""
    nseg = nstages + 1
    sn2 = (np.arange(1, nseg + 1) * snr_bound**2 / nseg).astype(np.float32)
    return np.sqrt(sn2[1:])


def trials_scheme(branching_pattern, trials_start: int = 1) -> np.ndarray:
    """Thresholds for one false alarm per stage's trials
    (``detection/schemes.py:53-75``)."""
    trials = np.cumprod(branching_pattern) * trials_start
    return stats.norm.isf(1 / trials)


def get_next_state(state_cur, threshold: float, success_h0: float, success_h1: float,
                   nbranches: float) -> np.void:
    """State after one stage (``thresholding.py:351-377``)."""
    nleaves_next = state_cur["complexity"] * nbranches
    nleaves_surv = nleaves_next * success_h0
    complexity_cumul = state_cur["complexity_cumul"] + nleaves_next
    success_h1_cumul = state_cur["success_h1_cumul"] * success_h1
    s = np.zeros(1, dtype=state_dtype)[0]
    s["success_h0"] = success_h0
    s["success_h1"] = success_h1
    s["complexity"] = nleaves_surv
    s["complexity_cumul"] = complexity_cumul
    s["success_h1_cumul"] = success_h1_cumul
    s["nbranches"] = nbranches
    s["threshold"] = threshold
    with np.errstate(divide="ignore", invalid="ignore"):
        s["cost"] = complexity_cumul / success_h1_cumul
    s["threshold_prev"] = state_cur["threshold"]
    s["success_h1_cumul_prev"] = state_cur["success_h1_cumul"]
    return s


def initial_state() -> np.void:
    s = np.ones(1, dtype=state_dtype)[0]
    s["threshold"] = -1.0
    s["threshold_prev"] = -1.0
    s["is_empty"] = False
    return s


def neighbouring_indices(beam_indices: np.ndarray, target_idx: int, num: int) -> np.ndarray:
    """``num`` beam entries around ``target_idx`` (``thresholding.py:27-43``)."""
    t = int(np.searchsorted(beam_indices, target_idx))
    left = max(0, t - num // 2)
    right = min(len(beam_indices), left + num)
    left = max(0, right - num)
    return beam_indices[left:right]


class FoldSim:
    """Batched fold simulation + scoring on one device.

    ``run(sets, var_cur)`` simulates every set in one launch. A set is
    ``(src, bias)``: ``src`` a device tensor of previous folds (or None for
    zeros), ``bias`` the template S/N; its output has ``n_prev *
    ceil(ntrials / n_prev)`` rows as in ``simulate_folds``."""

    def __init__(self, profile: np.ndarray, ntrials: int, ducy_max: float, wtsp: float, *,
                 seed: int = 0, device=None) -> None:
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._lib = _lib.load()
        self.nbins = len(profile)
        self.ntrials = int(ntrials)
        self.profile = torch.as_tensor(np.asarray(profile, np.float32)).to(self.device)
        self.widths = generate_box_width_trials(self.nbins, ducy_max=ducy_max, wtsp=wtsp)
        self.spec = _lib.score_spec(self.widths, self.nbins, 1.0, mode=1)
        self.seed = int(seed)
        self.calls = 0
        self.launches = 0

    def _stream(self) -> int:
        return _lib.stream_ptr(torch.cuda.current_stream(self.device))

    def run(self, sets: list[tuple[torch.Tensor | None, float]], var_add: float,
            var_next: float) -> tuple[list[torch.Tensor], list[np.ndarray]]:
        """Simulated folds (device) and their scores (host) per set."""
        nb = self.nbins
        srcs, counts, rows = [], [], []
        base = 0
        for src, _ in sets:
            n_prev = self.ntrials if src is None else int(src.shape[0])
            if n_prev == 0:
                msg = "No trials in the input folds"
                raise ValueError(msg)
            n_sim = n_prev * int(np.ceil(self.ntrials / n_prev))
            counts.append(n_sim)
            if src is not None:
                srcs.append(src)
                rows.append(base + np.arange(n_sim) % n_prev)
                base += n_prev
            else:
                rows.append(None)
        total = int(sum(counts))
        bias = np.concatenate([np.full(c, b, np.float32) for c, (_, b) in zip(counts, sets,
                                                                               strict=True)])
        dev = self.device
        any_src = bool(srcs)
        if any_src and any(r is None for r in rows):
            msg = "sets must all have sources or all start from zeros"
            raise ValueError(msg)
        folds_in = torch.cat(srcs).contiguous() if any_src else None
        src_row = (torch.from_numpy(np.concatenate(rows).astype(np.int64)).to(dev)
                   if any_src else None)
        bias_d = torch.from_numpy(bias).to(dev)
        out = torch.empty((total, nb), dtype=torch.float32, device=dev)
        scores = torch.empty(total, dtype=torch.float32, device=dev)
        seed = (self.seed * 0x9E3779B97F4A7C15 + self.calls) & 0xFFFFFFFFFFFFFFFF
        self.calls += 1
        _lib.check(self._lib.loki_sim_score_folds(
            _lib.ptr(folds_in), _lib.ptr(src_row), _lib.ptr(bias_d), total,
            _lib.ptr(self.profile), nb, float(np.sqrt(var_add)),
            float(np.sqrt(np.float32(var_next))),
            C.c_uint64(seed), self.spec, _lib.ptr(out), _lib.ptr(scores), self._stream()))
        self.launches += 1
        sc = scores.cpu().numpy()
        folds, host = [], []
        o = 0
        for c in counts:
            folds.append(out[o:o + c])
            host.append(sc[o:o + c])
            o += c
        return folds, host

    def run_bank(self, bank: torch.Tensor, offs: np.ndarray, cnts: np.ndarray,
                 biases: np.ndarray, var_add: float, var_next: float, *,
                 host_scores: bool = True) -> tuple[torch.Tensor, object, np.ndarray,
                                                    np.ndarray]:
        """``run`` for sets given as row ranges [offs, offs + cnts) of one bank:
        returns the simulated rows, their scores (host, or the device tensor
        with ``host_scores=False``) and each set's output offsets and counts."""
        cnts = np.asarray(cnts, np.int64)
        if np.any(cnts <= 0):
            msg = "No trials in the input folds"
            raise ValueError(msg)
        n_sim = cnts * np.ceil(self.ntrials / cnts).astype(np.int64)
        out_off = np.concatenate([[0], np.cumsum(n_sim)[:-1]]).astype(np.int64)
        total = int(n_sim.sum())
        set_of_row = np.repeat(np.arange(len(cnts)), n_sim)
        local = np.arange(total, dtype=np.int64) - out_off[set_of_row]
        src_row = np.asarray(offs, np.int64)[set_of_row] + local % cnts[set_of_row]
        bias = np.asarray(biases, np.float32)[set_of_row]
        dev = self.device
        src_d = torch.from_numpy(src_row).to(dev)
        bias_d = torch.from_numpy(bias).to(dev)
        out = torch.empty((total, self.nbins), dtype=torch.float32, device=dev)
        scores = torch.empty(total, dtype=torch.float32, device=dev)
        seed = (self.seed * 0x9E3779B97F4A7C15 + self.calls) & 0xFFFFFFFFFFFFFFFF
        self.calls += 1
        _lib.check(self._lib.loki_sim_score_folds(
            _lib.ptr(bank), _lib.ptr(src_d), _lib.ptr(bias_d), total, _lib.ptr(self.profile),
            self.nbins, float(np.sqrt(var_add)), float(np.sqrt(np.float32(var_next))),
            C.c_uint64(seed), self.spec, _lib.ptr(out), _lib.ptr(scores), self._stream()))
        self.launches += 1
        return out, (scores.cpu().numpy() if host_scores else scores), out_off, n_sim

    def take(self, folds: torch.Tensor, idx: np.ndarray) -> torch.Tensor:
        """Rows ``idx`` of ``folds`` (survivor compaction, one launch)."""
        n = len(idx)
        out = torch.empty((n, self.nbins), dtype=torch.float32, device=self.device)
        if n:
            idx_d = torch.from_numpy(np.ascontiguousarray(idx, np.int64)).to(self.device)
            _lib.check(self._lib.loki_gather_rows(_lib.ptr(folds.contiguous()), _lib.ptr(idx_d),
                                                  n, self.nbins, _lib.ptr(out), self._stream()))
            self.launches += 1
        return out


class _FoldState:
    """Surviving H0/H1 folds of a state and the noise variance they carry."""

    def __init__(self, h0, h1, variance: float, s0=None, s1=None) -> None:
        self.h0, self.h1, self.variance = h0, h1, variance
        self.s0, self.s1 = s0, s1  # scores, when already simulated

    @property
    def is_empty(self) -> bool:
        return self.h0 is None or self.h1 is None or self.h0.shape[0] == 0 \
            or self.h1.shape[0] == 0


def _path(sim: FoldSim, thresholds, branching_pattern, bias_snr, mode: str,
          survive_probs=None) -> np.ndarray:
    """Shared stage loop of evaluate_scheme / determine_scheme."""
    nstages = len(branching_pattern)
    var = 1.0
    (h0, h1), _ = sim.run([(None, 0.0), (None, bias_snr)], var_add=1.0, var_next=1.0)
    state = initial_state()
    out = []
    for istage in range(nstages):
        if h0.shape[0] == 0 or h1.shape[0] == 0:
            break  # path not viable: no trials survived
        (f0, f1), (s0, s1) = sim.run([(h0, 0.0), (h1, bias_snr)], var_add=1.0,
                                     var_next=var + 1.0)
        var += 1.0
        if mode == "prob":  # prune_folds_survival (thresholding.py:138-158)
            n_surv = int(survive_probs[istage] * len(s0))
            order = np.flip(np.argsort(s0, kind="stable"))[:n_surv]
            thr = float(s0[order[-1]]) if n_surv else float("inf")
            keep0 = order
        else:
            thr = float(thresholds[istage])
            keep0 = np.flatnonzero(s0 > thr)
        keep1 = np.flatnonzero(s1 > thr)
        state = get_next_state(state, thr, len(keep0) / len(s0), len(keep1) / len(s1),
                               float(branching_pattern[istage]))
        out.append(state)
        h0, h1 = sim.take(f0, keep0), sim.take(f1, keep1)
    return np.array(out, dtype=state_dtype)


def evaluate_scheme(thresholds, branching_pattern, ref_ducy: float, nbins: int = 64,
                    ntrials: int = 2048, snr_final: float = 8, ducy_max: float = 0.2,
                    wtsp: float = 1.0, *, seed: int = 0, device=None) -> np.ndarray:
    """States of a given threshold scheme (``thresholding.py:1062-1110``):
    one record per stage (``state_dtype``)."""
    nstages = len(branching_pattern)
    if len(thresholds) != nstages:
        msg = "Number of thresholds must match the number of stages"
        raise ValueError(msg)
    sim = FoldSim(generate_folded_profile(nbins=nbins, ducy=ref_ducy), ntrials, ducy_max, wtsp,
                  seed=seed, device=device)
    return _path(sim, thresholds, branching_pattern, snr_final / np.sqrt(nstages + 1), "thr")


def determine_scheme(survive_probs, branching_pattern, ref_ducy: float, nbins: int = 64,
                     ntrials: int = 2048, snr_final: float = 8, ducy_max: float = 0.2,
                     wtsp: float = 1.0, *, seed: int = 0, device=None) -> np.ndarray:
    """Thresholds that keep the given H0 survival fraction at each stage
    (``thresholding.py:1010-1059``)."""
    nstages = len(branching_pattern)
    if len(survive_probs) != nstages:
        msg = "Number of survive_probs must match the number of stages"
        raise ValueError(msg)
    sim = FoldSim(generate_folded_profile(nbins=nbins, ducy=ref_ducy), ntrials, ducy_max, wtsp,
                  seed=seed, device=device)
    return _path(sim, None, branching_pattern, snr_final / np.sqrt(nstages + 1), "prob",
                 survive_probs)


class DynamicThresholdScheme:
    """Dynamic-programming threshold design (``thresholding.py:702-1008``).

    ``states[istage, ithres, iprob]`` keeps, per threshold and bin of the
    cumulative H1 survival probability, the path of least cumulative
    complexity; ``run`` fills stages 1.. from stage 0 built at construction.
    ``mode="improved"`` simulates each surviving fold set once per stage and
    reuses it for every threshold; ``"legacy"`` simulates per transition.
    """

    def __init__(self, branching_pattern, ref_ducy: float, nbins: int = 64, ntrials: int = 1024,
                 nprobs: int = 10, prob_min: float = 0.05, snr_final: float = 8,
                 nthresholds: int = 100, ducy_max: float = 0.2, wtsp: float = 1.0,
                 beam_width: float = 0.7, mode: Literal["legacy", "improved"] = "legacy", *,
                 seed: int = 0, device=None) -> None:
        if mode not in ("legacy", "improved"):
            msg = f"mode must be 'legacy' or 'improved', got {mode!r}"
            raise ValueError(msg)
        self.mode = mode
        self.branching_pattern = np.asarray(branching_pattern)
        self.ref_ducy = ref_ducy
        self.profile = generate_folded_profile(nbins=nbins, ducy=ref_ducy)
        self.ntrials = ntrials
        self.snr_final = snr_final
        self.ducy_max = ducy_max
        self.wtsp = wtsp
        self.beam_width = beam_width
        self.thresholds = np.linspace(0.1, self.snr_final, nthresholds)
        self.prob_min = prob_min
        self.probs = np.logspace(np.log10(prob_min), 0, nprobs)
        empty = np.ones(1, dtype=state_dtype)[0]
        empty["threshold"] = -1.0
        empty["threshold_prev"] = -1.0
        self.states = np.full((self.nstages, self.nthresholds, self.nprobs), empty)
        # A cumulative branching of 1 gives trials_scheme = isf(1) = -inf, whose
        # beam (guess +- beam_width) holds no threshold and ends the design at
        # that stage; the guess is held at the lowest threshold instead.
        self.guess_path = np.maximum(
            np.minimum(bound_scheme(self.nstages, self.snr_final),
                       trials_scheme(self.branching_pattern, trials_start=1)),
            self.thresholds[0])
        self.sim = FoldSim(self.profile, ntrials, ducy_max, wtsp, seed=seed, device=device)
        self.folds_in: dict[tuple[int, int], _FoldState] = {}
        self._init_stage0()

    @property
    def nstages(self) -> int:
        return len(self.branching_pattern)

    @property
    def bias_snr(self) -> float:
        return self.snr_final / np.sqrt(self.nstages + 1)

    @property
    def nthresholds(self) -> int:
        return len(self.thresholds)

    @property
    def nprobs(self) -> int:
        return len(self.probs)

    @property
    def nbins(self) -> int:
        return len(self.profile)

    def get_current_thresholds_idx(self, istage: int) -> np.ndarray:
        guess = self.guess_path[istage]
        lo = max(0, guess - self.beam_width)
        hi = min(self.snr_final, guess + self.beam_width)
        return np.where((self.thresholds >= lo) & (self.thresholds <= hi))[0]

    def _iprob(self, s) -> int:
        return int(np.digitize(s["success_h1_cumul"], self.probs)) - 1

    def _transition(self, prev, sim_state: _FoldState, thr: float, nbranches: float):
        k0 = np.flatnonzero(sim_state.s0 > thr)
        k1 = np.flatnonzero(sim_state.s1 > thr)
        s = get_next_state(prev, thr, len(k0) / len(sim_state.s0), len(k1) / len(sim_state.s1),
                           nbranches)
        return s, (sim_state, k0, k1)

    def _materialise(self, pending) -> dict[tuple[int, int], _FoldState]:
        out = {}
        for key, (sim_state, k0, k1) in pending.items():
            out[key] = _FoldState(self.sim.take(sim_state.h0, k0),
                                  self.sim.take(sim_state.h1, k1), sim_state.variance)
        return out

    def _init_stage0(self) -> None:
        sim = self.sim
        (h0, h1), _ = sim.run([(None, 0.0), (None, self.bias_snr)], var_add=1.0, var_next=1.0)
        state = initial_state()
        beam = self.get_current_thresholds_idx(0)
        pending = {}
        if self.mode == "improved":
            (f0, f1), (s0, s1) = sim.run([(h0, 0.0), (h1, self.bias_snr)], 1.0, 2.0)
            shared = _FoldState(f0, f1, 2.0, s0, s1)
            per = {int(i): shared for i in beam}
        else:  # legacy: a fresh simulation per threshold
            sets = [s for _ in beam for s in ((h0, 0.0), (h1, self.bias_snr))]
            folds, scores = sim.run(sets, 1.0, 2.0)
            per = {int(i): _FoldState(folds[2 * n], folds[2 * n + 1], 2.0, scores[2 * n],
                                      scores[2 * n + 1]) for n, i in enumerate(beam)}
        for ithres in beam:
            cur, fold = self._transition(state, per[int(ithres)], float(self.thresholds[ithres]),
                                         float(self.branching_pattern[0]))
            iprob = self._iprob(cur)
            if iprob < 0:
                continue
            self.states[0, ithres, iprob] = cur
            pending[(int(ithres), iprob)] = fold
        self.folds_in = self._materialise(pending)

    def run(self, thres_neigh: int = 11) -> None:
        """Fill every stage after the first (``thresholding.py:904-963``).

        Each stage simulates all its fold sets in one launch, evaluates every
        (threshold, neighbour, probability bin) transition at once from the
        sorted scores, keeps per (threshold, bin) the first transition of least
        cumulative complexity in the reference's loop order, and compacts the
        winners' survivors with one gather."""
        for istage in range(1, self.nstages):
            self._stage(istage, thres_neigh)

    def _bank_of(self) -> tuple[torch.Tensor, dict]:
        """The current fold states as one bank and (h0, h1) row ranges."""
        keys = sorted(self.folds_in)
        parts, ranges, o = [], {}, 0
        for key in keys:
            fs = self.folds_in[key]
            if fs.is_empty:
                continue
            parts += [fs.h0, fs.h1]
            ranges[key] = (o, fs.h0.shape[0], o + fs.h0.shape[0], fs.h1.shape[0])
            o += fs.h0.shape[0] + fs.h1.shape[0]
        bank = torch.cat(parts).contiguous() if parts else None
        return bank, ranges

    def _stage(self, istage: int, thres_neigh: int) -> None:
        beam_cur = self.get_current_thresholds_idx(istage)
        beam_prev = self.get_current_thresholds_idx(istage - 1)
        prev = self.states[istage - 1]
        bank, ranges = self._bank_of()
        keys = [(int(j), k) for j in beam_prev for k in range(self.nprobs)
                if not prev[j, k]["is_empty"] and (int(j), k) in ranges]
        if not keys:
            self.folds_in = {}
            return
        kidx = {key: n for n, key in enumerate(keys)}
        # candidates in the reference's loop order: ithres, neighbour j, kprob
        c_thr, c_key = [], []
        for ithres in beam_cur:
            for j in neighbouring_indices(beam_prev, int(ithres), thres_neigh):
                for k in range(self.nprobs):
                    n = kidx.get((int(j), k))
                    if n is not None:
                        c_thr.append(int(ithres))
                        c_key.append(n)
        if not c_thr:
            self.folds_in = {}
            return
        c_thr = np.asarray(c_thr, np.int64)
        c_key = np.asarray(c_key, np.int64)
        # one simulation per key (improved) or per candidate (legacy)
        c_sim = c_key if self.mode == "improved" else np.arange(len(c_thr))
        sim_key = np.arange(len(keys)) if self.mode == "improved" else c_key
        offs, cnts, biases = [], [], []
        for n in sim_key:
            o0, n0, o1, n1 = ranges[keys[int(n)]]
            offs += [o0, o1]
            cnts += [n0, n1]
            biases += [0.0, self.bias_snr]
        var = self.folds_in[keys[0]].variance
        out, scores_d, out_off, n_sim = self.sim.run_bank(bank, np.array(offs), np.array(cnts),
                                                          np.array(biases), 1.0, var + 1.0,
                                                          host_scores=False)
        dev = self.sim.device
        # scores as a padded (set, row) matrix on the device (-inf pads)
        maxlen = int(n_sim.max())
        col = torch.arange(maxlen, device=dev)
        off_d = torch.from_numpy(out_off).to(dev)
        nsim_d = torch.from_numpy(n_sim).to(dev)
        valid = col[None, :] < nsim_d[:, None]
        pos = (off_d[:, None] + col[None, :]).clamp_max(scores_d.numel() - 1)
        smat = torch.where(valid, scores_d[pos], torch.full((), float("-inf"), device=dev))
        # survival of every candidate at its threshold, H0 and H1
        thr_c = self.thresholds[c_thr]
        thr_d = torch.from_numpy(thr_c.astype(np.float32)).to(dev)
        sets = torch.from_numpy(np.stack([2 * c_sim, 2 * c_sim + 1])).to(dev)  # (2, ncand)
        above = (smat[sets] > thr_d[None, :, None]).sum(dim=2)
        succ = (above.double() / nsim_d[sets].double()).cpu().numpy()
        # next states (get_next_state, vectorised; float32 fields as stored)
        pj = np.array([keys[int(n)] for n in c_key])
        pst = prev[pj[:, 0], pj[:, 1]]
        nbr = float(self.branching_pattern[istage])
        nleaves_next = pst["complexity"].astype(np.float64) * nbr
        cc64 = pst["complexity_cumul"].astype(np.float64) + nleaves_next
        sh64 = pst["success_h1_cumul"].astype(np.float64) * succ[1]
        cc = cc64.astype(np.float32)
        sh1c = sh64.astype(np.float32)
        iprob = np.digitize(sh1c, self.probs) - 1
        ok = np.flatnonzero((iprob >= 0) & (iprob < self.nprobs))
        # per (ithres, iprob): the first candidate (loop order) of least complexity
        grp = c_thr[ok] * self.nprobs + iprob[ok]
        srt = np.lexsort((ok, cc[ok], grp))
        first = np.unique(grp[srt], return_index=True)[1]
        winners = ok[srt[first]]
        if not len(winners):
            self.folds_in = {}
            return
        st = np.zeros(len(winners), dtype=state_dtype)
        st["success_h0"], st["success_h1"] = succ[0, winners], succ[1, winners]
        st["complexity"] = nleaves_next[winners] * succ[0, winners]
        st["complexity_cumul"] = cc[winners]
        st["success_h1_cumul"] = sh1c[winners]
        st["nbranches"] = nbr
        st["threshold"] = thr_c[winners]
        with np.errstate(divide="ignore", invalid="ignore"):
            st["cost"] = cc64[winners] / sh64[winners]
        st["threshold_prev"] = pst["threshold"][winners]
        st["success_h1_cumul_prev"] = pst["success_h1_cumul"][winners]
        st["is_empty"] = False
        self.states[istage, c_thr[winners], iprob[winners]] = st
        # survivors of the winners, H0 then H1 each, compacted in one gather
        wsets = torch.from_numpy(np.stack([2 * c_sim[winners], 2 * c_sim[winners] + 1],
                                          axis=1).reshape(-1)).to(dev)
        wthr = torch.from_numpy(np.repeat(thr_c[winners].astype(np.float32), 2)).to(dev)
        keep = smat[wsets] > wthr[:, None]
        counts = keep.sum(dim=1).cpu().numpy()
        r, cidx = torch.nonzero(keep, as_tuple=True)
        rows = off_d[wsets[r]] + cidx
        newbank = out[rows]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        self.folds_in = {}
        for n, w in enumerate(winners):
            o0, n0 = int(starts[2 * n]), int(counts[2 * n])
            o1, n1 = int(starts[2 * n + 1]), int(counts[2 * n + 1])
            self.folds_in[(int(c_thr[w]), int(iprob[w]))] = _FoldState(
                newbank[o0:o0 + n0], newbank[o1:o1 + n1], var + 1.0)

    def best_path(self) -> np.ndarray:
        """Thresholds of the least-cost final state, traced back stage by stage
        through ``threshold_prev`` / ``success_h1_cumul_prev``."""
        last = self.states[-1]
        ok = ~last["is_empty"]
        if not ok.any():
            return np.zeros(0, np.float32)
        cost = np.where(ok, last["cost"], np.inf)
        i, k = np.unravel_index(int(np.argmin(cost)), cost.shape)
        path = [float(last[i, k]["threshold"])]
        s = last[i, k]
        for istage in range(self.nstages - 2, -1, -1):
            cand = self.states[istage]
            m = (~cand["is_empty"]) & np.isclose(cand["threshold"], s["threshold_prev"]) & \
                np.isclose(cand["success_h1_cumul"], s["success_h1_cumul_prev"])
            if not m.any():
                break
            i, k = np.argwhere(m)[0]
            s = cand[i, k]
            path.append(float(s["threshold"]))
        return np.array(path[::-1], np.float32)

    def backtrack_best(self, min_probs: list[float] | None = None) -> list[np.ndarray]:
        """Least-cost complete schemes reaching each ``min_probs`` H1 survival
        (``detection/schemes.py:225-277``); see :func:`backtrack_best`."""
        return backtrack_best(self.states, self.thresholds, self.probs, min_probs)

    def save(self, outdir: str = ".") -> str:
        """The design as the reference's HDF5 file (``thresholding.py:965-1008``):
        attributes ntrials, snr_final, ref_ducy, ducy_max, wtsp, beam_width,
        mode, and datasets branching_pattern, profile, thresholds, probs,
        guess_path and states (``state_dtype`` records)."""
        from pyloki_gb300 import h5

        fb = (f"dynscheme_nstages_{self.nstages:03d}_nthresh_{self.nthresholds:03d}_"
              f"nprobs_{self.nprobs:03d}_ntrials_{self.ntrials:04d}_snr_{self.snr_final:04.1f}_"
              f"ducy_{self.ref_ducy:04.2f}_beam_{self.beam_width:03.1f}")
        path = Path(outdir) / f"{fb}.h5"
        with h5.File(path, "w") as f:
            f.attrs.update({"ntrials": np.int64(self.ntrials),
                            "snr_final": float(self.snr_final), "ref_ducy": float(self.ref_ducy),
                            "ducy_max": float(self.ducy_max), "wtsp": float(self.wtsp),
                            "beam_width": float(self.beam_width), "mode": str(self.mode)})
            for name in ("branching_pattern", "profile", "thresholds", "probs", "guess_path",
                         "states"):
                f.create_dataset(name, data=np.asarray(getattr(self, name)))
        return path.as_posix()


class DynamicThresholdSchemeAnalyser:
    """A saved design read back (``detection/schemes.py:614-660``
    ``DynamicThresholdSchemeAnalyser.from_file``): its states, thresholds,
    probability bins, branching pattern, guess path and beam width, and the
    best-path backtrack over them."""

    def __init__(self, states, thresholds, probs, branching_pattern, guess_path,
                 beam_width: float) -> None:
        self.states = np.asarray(states)
        self.thresholds = np.asarray(thresholds)
        self.probs = np.asarray(probs)
        self.branching_pattern = np.asarray(branching_pattern)
        self.guess_path = np.asarray(guess_path)
        self.beam_width = float(beam_width)

    @classmethod
    def from_file(cls, filename: str) -> DynamicThresholdSchemeAnalyser:
        from pyloki_gb300 import h5

        f = h5.read_file(filename)
        return cls(f["states"].data, f["thresholds"].data, f["probs"].data,
                   f["branching_pattern"].data, f["guess_path"].data, f.attrs["beam_width"])

    def backtrack_best(self, min_probs: list[float] | None = None) -> list[np.ndarray]:
        return backtrack_best(self.states, self.thresholds, self.probs, min_probs)


def backtrack_best(states: np.ndarray, thresholds: np.ndarray, probs: np.ndarray,
                   min_probs: list[float] | None = None) -> list[np.ndarray]:
    """Best threshold paths of a finished design
    (``DynamicThresholdSchemeAnalyser.backtrack_best``, ``detection/schemes.py:225-277``).

    For each ``min_prob``: among the non-empty final states whose cumulative
    H1 survival is at least ``min_prob``, the one of least ``cost``, traced
    back stage by stage to the state at (nearest threshold to
    ``threshold_prev``, probability bin of ``success_h1_cumul_prev``). Each
    result is the path's states (``state_dtype``, one per stage; its
    ``threshold`` field is the scheme), empty when no final state qualifies.
    Raises ``ValueError`` when the design has no complete scheme or the trace
    reaches an empty state.
    """
    if min_probs is None:
        min_probs = [probs[0]]
    final = states[-1]
    cloud = final[~final["is_empty"]]
    if len(cloud) == 0:
        msg = "No non-empty final states to plot"
        raise ValueError(msg)
    nstages = states.shape[0]
    out = []
    for min_prob in min_probs:
        ok = cloud[cloud["success_h1_cumul"] >= min_prob]
        if len(ok) == 0:
            out.append(np.zeros(0, dtype=states.dtype))
            continue
        path = [ok[np.argmin(ok["cost"])]]
        for istage in range(nstages - 2, -1, -1):
            prev_thr = path[0]["threshold_prev"]
            prev_prob = path[0]["success_h1_cumul_prev"]
            ithres = np.argmin(np.abs(thresholds - prev_thr))
            iprob = np.digitize(prev_prob, probs) - 1
            if iprob < 0 or states[istage, ithres, iprob]["is_empty"]:
                msg = (f"Backtracking failed at stage {istage} for threshold {prev_thr} "
                       f"and success probability {prev_prob}")
                raise ValueError(msg)
            path.insert(0, states[istage, ithres, iprob])
        out.append(np.array(path, dtype=states.dtype))
    return out


__all__ = ["DynamicThresholdScheme", "DynamicThresholdSchemeAnalyser", "FoldSim",
           "backtrack_best", "bound_scheme",
           "determine_scheme",
           "evaluate_scheme", "generate_folded_profile", "get_next_state",
           "neighbouring_indices", "state_dtype", "trials_scheme"]

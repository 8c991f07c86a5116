"""Learned branch proposal: a small MLP trained on the GPU by the library's
own tensor-core kernels (``loki_mlp_forward`` / ``loki_mlp_backward`` /
``loki_mlp_adam``).

The network maps 16 per-branch statistics of the pruning tree to the logit
of "this branch still has a descendant above threshold some levels later".
``Pruning`` can use it to order the parents of a level and, when a level
exceeds its budget, to expand the most promising parents first; the exact
per-level threshold still decides every emitted leaf, and without a model (or
within budget) pruning is the plain algorithm. The reference has no learned
part; nothing here changes results unless a budget is set.
"""

from __future__ import annotations

import numpy as np
import torch

from pyloki_gb300 import _lib

F = 16
H = 128
#: flat float32 parameter layout: name, shape
SHAPES = (("w1", (H, F)), ("b1", (H,)), ("w2", (H, H)), ("b2", (H,)), ("w3", (H,)),
          ("b3", (1,)))
_SIZES = [int(np.prod(s)) for _, s in SHAPES]
_OFFS = np.concatenate([[0], np.cumsum(_SIZES)]).astype(int)
NPARAMS = int(_OFFS[-1])


def init_params(seed: int = 0) -> np.ndarray:
    """PyTorch Linear default initialisation (uniform +-1/sqrt(fan_in))."""
    rng = np.random.default_rng(seed)
    parts = []
    for (name, shape), _ in zip(SHAPES, _SIZES, strict=True):
        fan_in = {"w1": F, "b1": F, "w2": H, "b2": H, "w3": H, "b3": H}[name]
        bound = 1.0 / np.sqrt(fan_in)
        parts.append(rng.uniform(-bound, bound, int(np.prod(shape))))
    return np.concatenate(parts).astype(np.float32)


class BranchMLP:
    """16 -> 128 -> 128 -> 1 ReLU network with bfloat16 weights and float32
    biases, accumulation and Adam state, resident on one GPU."""

    def __init__(self, params: np.ndarray | None = None, *, device=None, seed: int = 0) -> None:
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._lib = _lib.load()
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        if p.shape != (NPARAMS,):
            msg = f"expected {NPARAMS} parameters, got {p.shape}"
            raise ValueError(msg)
        dev = self.device
        self.params = torch.from_numpy(p.copy()).to(dev)
        self.grads = torch.zeros(NPARAMS + 1, dtype=torch.float32, device=dev)  # + loss
        self.m = torch.zeros(NPARAMS, dtype=torch.float32, device=dev)
        self.v = torch.zeros(NPARAMS, dtype=torch.float32, device=dev)
        self.wbf = torch.empty(NPARAMS, dtype=torch.bfloat16, device=dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.step = 0
        self._sync_bf16()

    # ---- layout ------------------------------------------------------------
    def _ptr(self, t: torch.Tensor, name: str) -> int:
        i = [n for n, _ in SHAPES].index(name)
        return t.data_ptr() + int(_OFFS[i]) * t.element_size()

    def _desc(self) -> _lib.LokiMLP:
        d = _lib.LokiMLP()
        d.w1, d.w2, d.w3 = (self._ptr(self.wbf, n) for n in ("w1", "w2", "w3"))
        d.b1, d.b2, d.b3 = (self._ptr(self.params, n) for n in ("b1", "b2", "b3"))
        return d

    def _grad_desc(self) -> _lib.LokiMLPGrad:
        g = _lib.LokiMLPGrad()
        for n, _ in SHAPES:
            setattr(g, n, self._ptr(self.grads, n))
        g.loss = self.grads.data_ptr() + NPARAMS * 4
        return g

    def _stream(self) -> int:
        return _lib.stream_ptr(torch.cuda.current_stream(self.device))

    def _sync_bf16(self) -> None:
        """bfloat16 copies of the weight matrices (biases stay float32)."""
        _lib.check(self._lib.loki_f32_to_bf16(self.params.data_ptr(), NPARAMS,
                                              self.wbf.data_ptr(), self._stream()))

    def _x(self, x) -> torch.Tensor:
        x = torch.as_tensor(x, dtype=torch.float32).to(self.device).contiguous()
        if x.ndim != 2 or x.shape[1] != F:
            msg = f"features must be (n, {F}), got {tuple(x.shape)}"
            raise ValueError(msg)
        return x

    # ---- inference and training --------------------------------------------
    def logits(self, x) -> torch.Tensor:
        x = self._x(x)
        out = torch.empty(x.shape[0], dtype=torch.float32, device=self.device)
        _lib.check(self._lib.loki_mlp_forward(self._desc(), x.data_ptr(), x.shape[0],
                                              out.data_ptr(), self.err.data_ptr(),
                                              self._stream()))
        return out

    def predict(self, x) -> torch.Tensor:
        """Survival probability of each branch."""
        return torch.sigmoid(self.logits(x))

    def loss_and_grads(self, x, y, wt=None, scale: float | None = None) -> tuple[float, torch.Tensor]:
        """Loss and the flat float32 gradient (a view of the accumulator)."""
        x = self._x(x)
        y = torch.as_tensor(y, dtype=torch.float32).to(self.device).contiguous()
        w = None if wt is None else torch.as_tensor(wt, dtype=torch.float32).to(
            self.device).contiguous()
        n = x.shape[0]
        scale = 1.0 / max(n, 1) if scale is None else scale
        self.grads.zero_()
        _lib.check(self._lib.loki_mlp_backward(
            self._desc(), x.data_ptr(), y.data_ptr(), 0 if w is None else w.data_ptr(), n,
            scale, self._grad_desc(), None, self.err.data_ptr(), self._stream()))
        return float(self.grads[NPARAMS]), self.grads[:NPARAMS]

    def train_step(self, x, y, wt=None, *, lr: float = 1e-3) -> float:
        loss, _ = self.loss_and_grads(x, y, wt)
        self.step += 1
        _lib.check(self._lib.loki_mlp_adam(self.params.data_ptr(), self.grads.data_ptr(),
                                           self.m.data_ptr(), self.v.data_ptr(), NPARAMS, lr,
                                           0.9, 0.999, 1e-8, self.step, self._stream()))
        self._sync_bf16()
        return loss

    def fit(self, x, y, wt=None, *, epochs: int = 10, batch: int = 8192, lr: float = 1e-3,
            seed: int = 0) -> list[float]:
        """Minibatch Adam over (x, y); returns the mean loss of each epoch."""
        x = self._x(x)
        y = torch.as_tensor(y, dtype=torch.float32).to(self.device)
        w = None if wt is None else torch.as_tensor(wt, dtype=torch.float32).to(self.device)
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(x.shape[0], generator=g).to(self.device)
            tot, cnt = 0.0, 0
            for s in range(0, x.shape[0], batch):
                idx = perm[s:s + batch]
                tot += self.train_step(x[idx], y[idx], None if w is None else w[idx],
                                       lr=lr) * len(idx)
                cnt += len(idx)
            hist.append(tot / max(cnt, 1))
        self.check_errors()
        return hist

    def check_errors(self) -> None:
        _lib.check_dev_err(self.err)

    def state(self) -> np.ndarray:
        return self.params.cpu().numpy()


# ---- branch statistics ------------------------------------------------------
def parent_features(prn, tree, level: int) -> torch.Tensor:
    """(n, 16) float32 statistics of the parents entering ``level``
    (``loki_branch_features``): score against the threshold they passed and
    the one their children face, the level, the score's z within the level
    and the shape of the normalised fold (peak, mean, spread)."""
    thr = prn.threshold_scheme
    n = tree.valid_size
    dev = tree.scores.device
    out = torch.empty((n, F), dtype=torch.float32, device=dev)
    if n == 0:
        return out
    folds = tree.folds
    if folds.is_complex():
        mag = folds.abs().float().contiguous()
        folds = mag
    std, mean = torch.std_mean(tree.scores.float()) if n > 1 else (
        torch.ones((), device=dev), tree.scores.float().mean())
    stats = torch.stack([mean, std]).contiguous()
    t_prev = float(thr[level - 2]) if level >= 2 else 0.0
    _lib.check(_lib.load().loki_branch_features(
        tree.scores.data_ptr(), folds.data_ptr(), n, folds.shape[-1], t_prev,
        float(thr[level - 1]), level / len(thr), 1.0 / float(np.sqrt(level + 1)),
        stats.data_ptr(), out.data_ptr(),
        _lib.stream_ptr(torch.cuda.current_stream(dev))))
    return out


class Recorder:
    """Parent hook that keeps the statistics of every parent of every level of
    a plain run; ``labels`` then marks the parents that lead to the run's best
    final leaves (or that are still alive some levels later) and returns every
    positive plus ``per_level`` random negatives of each level."""

    def __init__(self, per_level: int = 4096, seed: int = 0) -> None:
        self.per_level = per_level
        self.rng = np.random.default_rng(seed)
        self.samples: list[tuple[int, torch.Tensor]] = []
        self.sizes: list[int] = []

    def __call__(self, prn, tree, level: int):
        self.sizes.append(tree.valid_size)
        if tree.valid_size:
            self.samples.append((level, parent_features(prn, tree, level)))
        return None

    def labels(self, prn, lookahead: int, top_k: int | None = None
               ) -> tuple[torch.Tensor, torch.Tensor]:
        """Features and 0/1 labels of the finished run: a descendant among the
        last tree's ``top_k`` best leaves, or (``top_k`` None) a descendant
        ``lookahead`` levels later or in the last tree."""
        hist = [bt[:, 0].long().cpu().numpy() for bt in prn.backtrack_hist]
        last = len(hist)  # T_last: the deepest tree with survivors
        sizes = list(self.sizes) + [len(hist[-1]) if hist else 0]
        if top_k is not None:
            mark = np.zeros(sizes[last], bool)
            if sizes[last]:
                sc = prn.world_tree.scores.float().cpu().numpy()
                mark[np.argsort(-sc, kind="stable")[:top_k]] = True
            lab = [None] * (last + 1)
            lab[last] = mark
            for t in range(last - 1, -1, -1):
                m = np.zeros(sizes[t], bool)
                m[hist[t][lab[t + 1]]] = True
                lab[t] = m
        else:
            reach = [None] * (last + 1)
            reach[last] = np.full(sizes[last], last, np.int64)
            for t in range(last - 1, -1, -1):
                r = np.full(sizes[t], t, np.int64)
                np.maximum.at(r, hist[t], reach[t + 1])
                reach[t] = r
            lab = [reach[t] >= min(t + lookahead, last) for t in range(last + 1)]
        xs, ys = [], []
        for level, feats in self.samples:
            t = level - 1
            if t > last:
                continue
            y = lab[t]
            pos = np.flatnonzero(y)
            neg = np.flatnonzero(~y)
            if len(neg) > self.per_level:
                neg = self.rng.choice(neg, self.per_level, replace=False)
            if len(pos) > self.per_level:
                pos = self.rng.choice(pos, self.per_level, replace=False)
            idx = np.sort(np.concatenate([pos, neg]))
            it = torch.from_numpy(idx).to(feats.device)
            xs.append(feats[it])
            ys.append(torch.from_numpy(y[idx].astype(np.float32)).to(feats.device))
        self.samples = []
        if not xs:
            return torch.zeros((0, F)), torch.zeros(0)
        return torch.cat(xs), torch.cat(ys)


class BranchProposal:
    """Parent hook: when a level has more than ``budget`` parents, expand the
    ones the network ranks most likely to survive (ties at the cut are all
    kept); below the budget the level is the plain algorithm. With
    ``score_share`` > 0 that share of the budget goes to the highest-scoring
    parents whatever the network says, so strong paths are never dropped."""

    def __init__(self, net: BranchMLP, budget: int, score_share: float = 0.0) -> None:
        self.net = net
        self.budget = int(budget)
        self.score_share = float(score_share)
        self.levels_cut = 0

    def __call__(self, prn, tree, level: int):
        n = tree.valid_size
        if n <= self.budget:
            return None
        z = self.net.logits(parent_features(prn, tree, level))
        k_score = int(self.budget * self.score_share)
        k_net = self.budget - k_score
        keep = z >= torch.topk(z, k_net, sorted=False).values.min()
        if k_score:
            s = torch.nan_to_num(tree.scores, nan=float("-inf"))
            keep |= s >= torch.topk(s, k_score, sorted=False).values.min()
        self.levels_cut += 1
        return keep.to(torch.uint8)


def _prune_run(dyp_of, ts, cfg, thresholds, ref, hook, device, max_sugg, batch_size):
    """One pruning run over the FFA fold of ``ts``; returns (pruning, leaves, ms)."""
    from pyloki_gb300.prune import Pruning

    dyp = dyp_of(ts)
    prn = Pruning(dyp, thresholds, max_sugg=max_sugg, batch_size=batch_size)
    prn.parent_hook = hook
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    t0.record()
    prn.initialize(ref)
    for _ in range(dyp.nsegments - 1):
        prn.execute_iter()
        if prn.prune_complete:
            break
    prn._do_ascend()
    t1.record()
    torch.cuda.synchronize(device)
    leaves = sum(st.n_leaves for st in prn.pstats[1:])
    return prn, leaves, t0.elapsed_time(t1)


def study(cfg, thresholds, make_series, *, train_seeds, test_seeds, noise_seeds,
          budget, lookahead: int = 16, top_k: int | None = 64, per_level: int = 2048,
          epochs: int = 6, score_share: float = 0.0,
          det_snr: float = 8.0, max_sugg: int = 2**18, batch_size: int = 1024,
          device=None, seed: int = 0) -> dict:
    """Train the branch-survival network on statistics of plain pruning runs
    and compare learned-proposal pruning with plain pruning on held-out
    series.

    ``make_series(seed, inject)`` returns a TimeSeries (with an injected pulsar
    when ``inject``). Labels mark the sampled parents with a descendant among
    the run's ``top_k`` best final leaves (or, with ``top_k`` None, alive
    ``lookahead`` levels later). Recall is the fraction of held-out injected series whose
    best final score under the learned proposal is within 1e-3 of the plain
    run's; the false-alarm rate is the fraction of noise-only series whose
    best final score reaches ``det_snr`` (plain and learned)."""
    import time

    from pyloki_gb300.ffa import DynamicProgramming

    dev = torch.device(device) if device is not None else torch.device(
        "cuda", torch.cuda.current_device())

    def dyp_of(ts):
        d = DynamicProgramming(ts, cfg, device=dev)
        d.initialize()
        d.execute()
        return d

    ref = None
    xs, ys = [], []
    t_rec = time.perf_counter()
    for sd in train_seeds:
        ts = make_series(sd, True)
        rec = Recorder(per_level=per_level, seed=sd)
        d = dyp_of(ts)
        ref = d.nsegments // 2 if ref is None else ref
        prn, _, _ = _prune_run(lambda _t, d=d: d, ts, cfg, thresholds, ref, rec, dev,
                               max_sugg, batch_size)
        x, y = rec.labels(prn, lookahead, top_k)
        xs.append(x)
        ys.append(y)
    x = torch.cat(xs)
    y = torch.cat(ys)
    pos = float(y.mean())
    wt = torch.where(y > 0.5, 0.5 / max(pos, 1e-6), 0.5 / max(1 - pos, 1e-6))
    rec_s = time.perf_counter() - t_rec
    net = BranchMLP(device=dev, seed=seed)
    t_fit = time.perf_counter()
    hist = net.fit(x, y, wt, epochs=epochs, batch=8192, lr=2e-3, seed=seed)
    torch.cuda.synchronize(dev)
    fit_s = time.perf_counter() - t_fit
    with torch.no_grad():
        pred = net.predict(x) > 0.5
    train_acc = float((pred == (y > 0.5)).float().mean())

    def compare(seeds, inject, budgets):
        rows = []
        for sd in seeds:
            ts = make_series(sd, inject)
            d = dyp_of(ts)
            p0, l0, ms0 = _prune_run(lambda _t: d, ts, cfg, thresholds, ref, None, dev,
                                     max_sugg, batch_size)
            b0 = float(p0.world_tree.scores.max()) if p0.world_tree.valid_size else float("-inf")
            row = {"seed": int(sd), "plain_best": b0, "plain_leaves": int(l0), "plain_ms": ms0,
                   "learned": {}}
            for bud in budgets:
                prop = BranchProposal(net, bud, score_share)
                p1, l1, ms1 = _prune_run(lambda _t: d, ts, cfg, thresholds, ref, prop, dev,
                                         max_sugg, batch_size)
                b1 = (float(p1.world_tree.scores.max()) if p1.world_tree.valid_size
                      else float("-inf"))
                row["learned"][bud] = {"best": b1, "leaves": int(l1), "ms": ms1,
                                       "levels_cut": prop.levels_cut,
                                       "parents_skipped": int(p1.parents_skipped)}
            rows.append(row)
        return rows

    budgets = [int(b) for b in (budget if np.ndim(budget) else [budget])]
    # untimed warm-up of both paths (first launches of the MLP, feature and
    # selection kernels) on a series outside the evaluation
    warm = make_series(int(train_seeds[0]), True)
    dw = dyp_of(warm)
    _prune_run(lambda _t: dw, warm, cfg, thresholds, ref, None, dev, max_sugg, batch_size)
    _prune_run(lambda _t: dw, warm, cfg, thresholds, ref,
               BranchProposal(net, min(budgets), score_share), dev, max_sugg, batch_size)
    inj = compare(test_seeds, True, budgets)
    noise = compare(noise_seeds, False, budgets)
    rows = inj + noise
    l0 = sum(r["plain_leaves"] for r in rows)
    ms0 = sum(r["plain_ms"] for r in rows)
    per_budget = {}
    for bud in budgets:
        l1 = sum(r["learned"][bud]["leaves"] for r in rows)
        ms1 = sum(r["learned"][bud]["ms"] for r in rows)
        per_budget[str(bud)] = {
            "recall_vs_plain": float(np.mean([r["learned"][bud]["best"] >= r["plain_best"] - 1e-3
                                              for r in inj])) if inj else None,
            "false_alarm_learned": float(np.mean([r["learned"][bud]["best"] >= det_snr
                                                  for r in noise])) if noise else None,
            "learned_leaves_per_s": l1 / (ms1 * 1e-3),
            "plain_equivalent_leaves_per_s": l0 / (ms1 * 1e-3), "speedup": ms0 / ms1,
            "leaves_fraction": l1 / max(l0, 1),
        }
    ok = [b for b in budgets if inj and per_budget[str(b)]["recall_vs_plain"] >= 0.99]
    at99 = ({"budget": min(ok), **{k: per_budget[str(min(ok))][k]
                                   for k in ("recall_vs_plain", "speedup", "leaves_fraction")}}
            if ok else None)
    return {
        "at_recall_0.99": at99,
        "train_series": len(train_seeds), "train_samples": int(x.shape[0]),
        "positive_fraction": pos, "label": (f"ancestor of the final top {top_k}"
                                            if top_k else f"alive {lookahead} levels later"),
        "epochs": epochs, "loss_per_epoch": hist, "train_accuracy": train_acc,
        "record_s": rec_s, "fit_s": fit_s, "det_snr": det_snr, "score_share": score_share,
        "false_alarm_plain": float(np.mean([r["plain_best"] >= det_snr for r in noise]))
        if noise else None,
        "plain_leaves_per_s": l0 / (ms0 * 1e-3),
        "budgets": per_budget, "injected": inj, "noise": noise,
    }


__all__ = ["BranchMLP", "BranchProposal", "NPARAMS", "Recorder", "SHAPES", "init_params",
           "parent_features", "study"]

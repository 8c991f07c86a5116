"""Learned branch proposal: a small MLP trained on the GPU by the library's
own tensor-core kernels (``loki_mlp_forward`` / ``loki_mlp_backward`` /
``loki_mlp_adam``).

The network maps 16 per-branch statistics of the pruning tree to the logit
of "this branch still has a descendant above threshold some levels later".
``Pruning`` can use it to order the parents of a level and, when a level
exceeds its budget, to expand the most promising parents first; the exact
per-level threshold still judges every emitted leaf, and without a model (or
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

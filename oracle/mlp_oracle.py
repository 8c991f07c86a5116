"""CPU oracle of the branch-survival MLP (test infrastructure only).

Restates the network of ``pyloki_gb300/csrc/mlp.cu`` in float64 numpy with
the same bfloat16 rounding points as the tensor-core kernels: inputs and
weights rounded to bfloat16, hidden activations and back-propagated
gradients rounded to bfloat16 where they become MMA operands, biases and
accumulations in float32/float64. The loss is the weighted binary
cross-entropy with logits, ``scale * sum wt * (softplus(z) - y z)``.
The reference (pyloki) has no learned part, so this oracle is pinned only by
finite differences (``finite_difference``) and by the kernels' own test.
"""

from __future__ import annotations

import numpy as np

F, H = 16, 128
SHAPES = (("w1", (H, F)), ("b1", (H,)), ("w2", (H, H)), ("b2", (H,)), ("w3", (H,)),
          ("b3", (1,)))


def split(flat: np.ndarray) -> dict[str, np.ndarray]:
    """Parameter dict from the flat float32 layout [w1, b1, w2, b2, w3, b3]."""
    out, o = {}, 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + size], np.float32).reshape(shape)
        o += size
    return out


def nparams() -> int:
    return sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(a) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even) as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _f32(a) -> np.ndarray:
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def forward(p: dict, x: np.ndarray) -> dict:
    xb = bf16(x)
    w1, w2, w3 = bf16(p["w1"]), bf16(p["w2"]), bf16(p["w3"])
    z1 = _f32(xb @ w1.T)
    h1 = bf16(np.maximum(_f32(z1 + p["b1"].astype(np.float64)), 0.0))
    z2 = _f32(h1 @ w2.T)
    h2 = np.maximum(_f32(z2 + p["b2"].astype(np.float64)), 0.0)
    logit = h2 @ w3 + float(p["b3"][0])
    return {"xb": xb, "w1": w1, "w2": w2, "w3": w3, "h1": h1, "h2": h2, "logit": logit}


def softplus(z):
    return np.where(z > 0, z + np.log1p(np.exp(-np.abs(z))), np.log1p(np.exp(-np.abs(z))))


def loss_and_grads(flat: np.ndarray, x: np.ndarray, y: np.ndarray, wt=None,
                   scale: float = 1.0) -> tuple[float, dict, np.ndarray]:
    """Loss, gradients (dict of float64 arrays in the parameter shapes) and
    logits, with the kernels' rounding points."""
    p = split(flat)
    f = forward(p, x)
    wt = np.ones(len(x)) if wt is None else np.asarray(wt, np.float64)
    z = f["logit"]
    y = np.asarray(y, np.float64)
    loss = float(np.sum(scale * wt * (softplus(z) - y * z)))
    g = scale * wt * (1.0 / (1.0 + np.exp(-z)) - y)
    on2 = f["h2"] > 0
    dz2 = g[:, None] * f["w3"][None, :] * on2
    dz2b = bf16(dz2)
    dh1 = dz2b @ f["w2"]
    on1 = f["h1"] > 0
    dz1 = _f32(dh1) * on1
    dz1b = bf16(dz1)
    grads = {
        "w1": dz1b.T @ f["xb"], "b1": dz1.sum(0), "w2": dz2b.T @ f["h1"], "b2": dz2.sum(0),
        "w3": (g[:, None] * f["h2"]).sum(0), "b3": np.array([g.sum()]),
    }
    return loss, grads, z


def flatten(grads: dict) -> np.ndarray:
    return np.concatenate([np.asarray(grads[n], np.float64).reshape(-1) for n, _ in SHAPES])


def finite_difference(flat: np.ndarray, x, y, idx, eps=1e-3) -> np.ndarray:
    """Central differences of the float64 loss of an unrounded network
    (weights and activations left in float64) at the parameter indices idx,
    to pin the oracle's gradient expressions."""
    def loss_of(fl):
        p = split(fl.astype(np.float32))
        p = {k: v.astype(np.float64) for k, v in p.items()}
        h1 = np.maximum(x @ p["w1"].T + p["b1"], 0.0)
        h2 = np.maximum(h1 @ p["w2"].T + p["b2"], 0.0)
        z = h2 @ p["w3"] + p["b3"][0]
        return float(np.sum(softplus(z) - y * z))
    out = []
    for i in idx:
        a = flat.astype(np.float64).copy()
        b = a.copy()
        a[i] += eps
        b[i] -= eps
        out.append((loss_of(a) - loss_of(b)) / (2 * eps))
    return np.array(out)


def exact_grads(flat: np.ndarray, x, y) -> np.ndarray:
    """Analytic float64 gradients of the unrounded network (no bfloat16)."""
    p = {k: v.astype(np.float64) for k, v in split(flat).items()}
    z1 = x @ p["w1"].T + p["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ p["w2"].T + p["b2"]
    h2 = np.maximum(z2, 0.0)
    z = h2 @ p["w3"] + p["b3"][0]
    g = 1.0 / (1.0 + np.exp(-z)) - y
    dz2 = g[:, None] * p["w3"][None, :] * (h2 > 0)
    dz1 = (dz2 @ p["w2"]) * (h1 > 0)
    return flatten({"w1": dz1.T @ x, "b1": dz1.sum(0), "w2": dz2.T @ h1, "b2": dz2.sum(0),
                    "w3": (g[:, None] * h2).sum(0), "b3": np.array([g.sum()])})

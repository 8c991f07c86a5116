"""Tensor-core MLP kernels against the CPU oracle: logits, loss and every
gradient (bfloat16 operands, float32 accumulation), and training by the
library's own forward, backward and Adam kernels."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

# float32 accumulation order differs from the oracle's float64 sums, which
# can flip a bfloat16 rounding of a hidden activation; relative L2 errors
GRAD_REL_TOL = 2e-2
LOGIT_ABS_TOL = 2e-3


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, M.F)).astype(np.float32)
    y = (x[:, 0] + 0.5 * x[:, 1] * x[:, 2] > 0).astype(np.float32)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return x, y, w


@pytest.mark.parametrize("n", [1, 127, 1000, 40000])
def test_forward_matches_oracle(cuda_device, n):
    from pyloki_gb300.learned import BranchMLP, init_params

    flat = init_params(5)
    net = BranchMLP(flat, device=cuda_device)
    x, _, _ = _data(n, n)
    got = net.logits(x).cpu().numpy()
    net.check_errors()
    ref = M.forward(M.split(flat), x)["logit"]
    np.testing.assert_allclose(got, ref, atol=LOGIT_ABS_TOL, rtol=1e-3)


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_gradients_match_oracle(cuda_device, n):
    from pyloki_gb300.learned import BranchMLP, SHAPES, init_params

    flat = init_params(7)
    net = BranchMLP(flat, device=cuda_device)
    x, y, w = _data(n, 100 + n)
    loss, g = net.loss_and_grads(x, y, w, scale=1.0 / n)
    net.check_errors()
    rl, rg, _ = M.loss_and_grads(flat, x, y, w, scale=1.0 / n)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    g = g.cpu().numpy().astype(np.float64)
    o = 0
    for name, shape in SHAPES:
        size = int(np.prod(shape))
        got, ref = g[o:o + size], np.asarray(rg[name], np.float64).reshape(-1)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < GRAD_REL_TOL, (name, err)
        o += size


def test_training_reduces_loss_and_learns(cuda_device):
    from pyloki_gb300.learned import BranchMLP

    x, y, _ = _data(32768, 9)
    net = BranchMLP(device=cuda_device, seed=1)
    hist = net.fit(x, y, epochs=8, batch=4096, lr=3e-3)
    assert hist[-1] < 0.6 * hist[0]
    xt, yt, _ = _data(8192, 10)
    acc = ((net.predict(xt).cpu().numpy() > 0.5) == (yt > 0.5)).mean()
    assert acc > 0.9


def test_timeout_path_reports_and_recovers(cuda_device):
    """The MLP kernels' give-up path after a bounded tensor-core wait: with
    the test hook on, completed waits count as expired (nothing is left in
    flight), the kernels free their tensor memory and set
    LOKI_DEVERR_TIMEOUT, and the host raises LokiError. With the hook off
    the next forward pass is correct again."""
    from pyloki_gb300 import _lib
    from pyloki_gb300.learned import BranchMLP, init_params

    lib = _lib.load()
    flat = init_params(7)
    net = BranchMLP(flat, device=cuda_device)
    x, y, w = _data(300, 3)
    try:
        _lib.check(lib.loki_mlp_force_timeout(1))
        net.logits(x)
        with pytest.raises(_lib.LokiError, match="timed out"):
            net.check_errors()
        net.err.zero_()
        net.loss_and_grads(x, y, w)
        with pytest.raises(_lib.LokiError, match="timed out"):
            net.check_errors()
    finally:
        _lib.check(lib.loki_mlp_force_timeout(0))
    net.err.zero_()
    got = net.logits(x).cpu().numpy()
    net.check_errors()
    ref = M.forward(M.split(flat), x)["logit"]
    np.testing.assert_allclose(got, ref, atol=LOGIT_ABS_TOL, rtol=1e-3)

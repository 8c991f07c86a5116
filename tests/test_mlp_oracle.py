"""The MLP oracle (CPU): its gradient expressions against central finite
differences of the unrounded network, its bfloat16 rounding, and the flat
parameter layout shared with the GPU module."""

from __future__ import annotations

import numpy as np

from oracle import mlp_oracle as M


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, -2.5, 3.0e-39, 65504.0], np.float32)
    got = M.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0  # tie -> even
    assert got[2] == 1.0 + 2**-7
    assert got[3] == -2.5
    import torch

    np.testing.assert_array_equal(got, torch.from_numpy(x).to(torch.bfloat16).double().numpy())


def test_exact_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    flat = (rng.uniform(-1, 1, M.nparams()) * 0.2).astype(np.float32)
    x = rng.standard_normal((64, M.F))
    y = (rng.random(64) > 0.5).astype(float)
    idx = [0, 7, 2047, 2048 + 5, 2176 + 999, 2176 + 16384 + 3, M.nparams() - 2, M.nparams() - 1]
    fd = M.finite_difference(flat, x, y, idx, eps=1e-4)
    np.testing.assert_allclose(M.exact_grads(flat, x, y)[idx], fd, atol=1e-5, rtol=1e-4)


def test_rounded_oracle_close_to_exact_and_layout():
    from pyloki_gb300.learned import NPARAMS, SHAPES, init_params

    assert NPARAMS == M.nparams() and tuple(SHAPES) == tuple(M.SHAPES)
    rng = np.random.default_rng(1)
    flat = init_params(3)
    x = rng.standard_normal((256, M.F))
    y = (rng.random(256) > 0.5).astype(float)
    _, g, _ = M.loss_and_grads(flat, x, y)
    ex = M.exact_grads(flat, x, y)
    # bfloat16 operands move the gradient by a few percent, not more
    assert np.linalg.norm(M.flatten(g) - ex) / np.linalg.norm(ex) < 0.05

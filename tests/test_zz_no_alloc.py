"""loki_brutefold_noalloc: the brute fold with the library's fixed phase scratch.

Collected last on purpose: it must give the same folds as loki_brutefold
whether it runs alone or after every other test has used the device.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

TSAMP = 64e-6


def _noalloc(lib, te, tv, tf, seg, nbins, t_ref, out, stream):
    from pyloki_gb300 import _lib

    return lib.loki_brutefold_noalloc(_lib.ptr(te), _lib.ptr(tv), te.numel(), _lib.ptr(tf),
                                      tf.numel(), seg, nbins, TSAMP, t_ref, _lib.ptr(out),
                                      stream)


def test_noalloc_rejects_oversize_segment_without_a_gpu_call():
    """Argument checks run before any CUDA call (fake, never dereferenced pointers)."""
    from pyloki_gb300 import _lib

    try:
        lib = _lib.load()
    except RuntimeError:
        pytest.skip("libloki_gb300.so not built")
    cap = lib.loki_brutefold_noalloc_scratch_bytes()
    assert cap == 16 << 20
    fake = C.c_void_p(0x1000)
    for nbins, limit in [(64, cap), (300, cap // 2)]:
        rc = lib.loki_brutefold_noalloc(fake, fake, 4 * limit, fake, 8, limit + 1, nbins,
                                        TSAMP, 0.0, fake, None)
        assert rc == _lib.LOKI_ERR_CAPACITY
        assert b"no-alloc limit" in lib.loki_last_error()
    assert lib.loki_brutefold_noalloc(None, fake, 10, fake, 1, 4, 64, TSAMP, 0.0, fake,
                                      None) == _lib.LOKI_ERR_INVALID
    assert lib.loki_brutefold_noalloc(fake, fake, 10, fake, 1, 4, 1000, TSAMP, 0.0, fake,
                                      None) == _lib.LOKI_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_noalloc_matches_brutefold_on_consecutive_calls(cuda_device):
    """Two calls in a row (different grids and bin counts, several frequency
    chunks each because the map outgrows the fixed scratch) against
    loki_brutefold with its own scratch, plus the oracle on a slice."""
    import torch

    from pyloki_gb300 import _lib
    from pyloki_gb300.ffa import brutefold

    lib = _lib.load()
    stream = _lib.stream_ptr(torch.cuda.current_stream(cuda_device))
    rng = np.random.default_rng(11)
    seg = 1 << 16
    n = 4 * seg + 3000  # ragged last segment
    ts_e = rng.standard_normal(n).astype(np.float32)
    ts_v = (1 + rng.random(n)).astype(np.float32)
    te = torch.from_numpy(ts_e).to(cuda_device)
    tv = torch.from_numpy(ts_v).to(cuda_device)
    cases = [(64, np.linspace(40.0, 41.0, 600), 0.02),   # 256 freqs a chunk -> 3 chunks
             (300, np.linspace(3.0, 3.5, 300), 0.0)]     # 128 freqs a chunk -> 3 chunks
    nseg = -(-n // seg)
    for nbins, freqs, t_ref in cases:
        tf = torch.from_numpy(freqs).to(cuda_device)
        want = brutefold(te, tv, tf, seg, nbins, TSAMP, t_ref)
        got = torch.full((nseg, len(freqs), 2, nbins), float("nan"), device=cuda_device)
        _lib.check(_noalloc(lib, te, tv, tf, seg, nbins, t_ref, got, stream))
        torch.cuda.synchronize(cuda_device)
        np.testing.assert_array_equal(got.cpu().numpy(), want.cpu().numpy())
        sl = slice(0, len(freqs), 97)
        ref = O.brutefold(ts_e, ts_v, freqs[sl], seg, nbins, TSAMP, t_ref)
        np.testing.assert_array_equal(got[:, sl].cpu().numpy(), ref)

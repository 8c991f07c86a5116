"""Shared test helpers: the ``gpu`` marker, golden fixtures, configs."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libloki_gb300.so")


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as d:
        return {k: d[k] for k in d.files}


def cfg_from_golden(d: dict, **kw):
    from pyloki_gb300.config import PulsarSearchConfig

    return PulsarSearchConfig(
        nsamps=int(d["nsamps"]), tsamp=float(d["tsamp"]), nbins=int(d["nbins"]),
        eta=float(d["eta"]), param_limits=d["param_limits"], ducy_max=float(d["ducy_max"]),
        wtsp=float(d["wtsp"]), use_fourier=False, **kw)


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyloki_gb300 import _lib

    _lib.load()
    return torch.device("cuda", 0)

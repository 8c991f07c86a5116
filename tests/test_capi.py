"""The C-ABI library: it loads, and exports every entry point the header declares."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols() -> list[str]:
    names = []
    for hdr in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", hdr.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:int64_t|int|const char\*|void)\s+(loki_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from pyloki_gb300 import _lib, build

    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "loki_brutefold" in names and "loki_ffa_level" in names
    assert len(names) >= 9


def test_library_exports_declared_symbols(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_bindings_cover_header():
    from pyloki_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_error_string(lib):
    assert lib.loki_version() >= 1
    assert isinstance(lib.loki_last_error(), bytes)


def test_argument_validation_without_gpu(lib):
    """Invalid arguments are rejected on the host before any CUDA call."""
    from pyloki_gb300 import _lib

    rc = lib.loki_brutefold(None, None, 0, None, 0, 0, 64, 1e-3, 0.0, None, 0, None, None)
    assert rc == _lib.LOKI_ERR_INVALID
    assert b"null" in lib.loki_last_error()
    desc = _lib.LokiFFALevel()
    desc.nparams = 7
    rc = lib.loki_ffa_level(ctypes.byref(desc), None, None, None, None)
    assert rc == _lib.LOKI_ERR_INVALID
    with pytest.raises(ValueError):
        _lib.check(rc)
    spec = _lib.score_spec([1, 2, 4], 64)
    spec.wmax = 3
    rc = lib.loki_boxcar_snr(None, 10, 64, ctypes.byref(spec), None, None)
    assert rc == _lib.LOKI_ERR_INVALID


def test_score_spec_constants():
    import numpy as np

    from pyloki_gb300 import _lib

    sp = _lib.score_spec([1, 2, 4, 8], 64, stdnoise=2.0)
    assert sp.nwidths == 4 and sp.wmax == 8 and sp.inv_stdnoise == 0.5
    h = np.sqrt((64 - 8) / (64 * 8))
    b = 8 * h / (64 - 8)
    assert sp.hb[3] == h + b and sp.b[3] == b


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the C structs have the header's sizes and offsets."""
    import subprocess

    from pyloki_gb300 import _lib

    structs = [_lib.LokiFFALevel, _lib.LokiFFACoord, _lib.LokiScoreSpec,
               _lib.LokiPruneLevel, _lib.LokiBranchInfo, _lib.LokiPruneTree,
               _lib.LokiPruneWork, _lib.LokiPruneLevelStats, _lib.LokiPruneRun,
               _lib.LokiPruneJob, _lib.LokiAscendJob, _lib.LokiGatherPart,
               _lib.LokiSeedJob]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "loki_gb300.h"',
             "int main(void) {"]
    for st in structs:
        name = st.__name__
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in st._fields_:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True,
                                                       text=True, check=True).stdout.splitlines())
    for st in structs:
        name = st.__name__
        assert int(got[name]) == ctypes.sizeof(st), name
        for fname, _ in st._fields_:
            assert int(got[f"{name}.{fname}"]) == getattr(st, fname).offset, (name, fname)

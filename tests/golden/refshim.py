"""Stand-in modules that let the pure-Python body of pyloki's numba code run.

Used only by ``make_fixtures.py`` in a container that has the pyloki source
tree; nothing on the test or product path imports this module.

numba, llvmlite and astropy are not installed, so each ``@njit`` decorator is
replaced by the identity, ``prange`` by ``range`` and the structref machinery
by plain classes. The result runs the reference's algorithms with numpy/IEEE
semantics (no fastmath contraction), which is the semantics the CUDA kernels
and the C oracle reproduce.
"""

from __future__ import annotations

import importlib.metadata as _md
import sys
import time as _time
import types as _t

import numpy as np


def _deco(*a, **k):
    if len(a) == 1 and callable(a[0]) and not k:
        return a[0]
    return lambda f: f


class _Any:
    def __getattr__(self, n):
        return _Any()

    def __getitem__(self, k):
        return _Any()

    def __call__(self, *a, **k):
        return _Any()


def _vectorize(*a, **k):
    def wrap(f):
        otype = np.float64 if f.__name__ == "get_phase_idx" else np.int64
        v = np.vectorize(f, otypes=[otype])

        def call(*args):
            r = v(*args)
            return r.item() if np.ndim(r) == 0 else r

        return call

    if len(a) == 1 and callable(a[0]):
        return wrap(a[0])
    return wrap


class _StructRef:
    def __init__(self, fields=None):
        self.fields = fields


class _StructRefProxy:
    pass


_BOXED: dict = {}


def _define_boxing(tmpl, proxy):
    _BOXED[tmpl] = proxy
    for name, val in list(vars(proxy).items()):
        # A property whose getter only returns ``self.<same name>`` is a plain
        # field accessor; drop it so the instance attribute is used instead.
        if (
            isinstance(val, property)
            and val.fget is not None
            and val.fget.__code__.co_names == (name,)
        ):
            delattr(proxy, name)


def install(reference_src: str) -> None:
    """Install the stand-ins and put ``reference_src`` first on sys.path."""
    numba = _t.ModuleType("numba")
    numba.njit = _deco
    numba.jit = _deco
    numba.prange = range
    numba.vectorize = _vectorize
    ntypes = _Any()
    ntypes.StructRef = _StructRef
    ntypes.ExternalFunction = lambda name, sig: (
        lambda: int(_time.process_time() * 1e6)
    )
    numba.types = ntypes
    numba.typed = _t.SimpleNamespace(List=list)
    numba.core = _t.ModuleType("numba.core")
    numba.core.types = ntypes
    numba.core.typing = _Any()
    exp = _t.ModuleType("numba.experimental")
    sr = _t.ModuleType("numba.experimental.structref")
    sr.StructRefProxy = _StructRefProxy
    sr.register = lambda cls: cls
    sr.define_boxing = _define_boxing
    sr.new = lambda typ: object.__new__(_BOXED[type(typ)])
    exp.structref = sr
    ext = _t.ModuleType("numba.extending")
    ext.overload = lambda *a, **k: (lambda f: f)
    ext.overload_method = lambda *a, **k: (lambda f: f)
    for name, mod in {
        "numba": numba,
        "numba.experimental": exp,
        "numba.experimental.structref": sr,
        "numba.extending": ext,
        "numba.core": numba.core,
    }.items():
        sys.modules[name] = mod
    astropy = _t.ModuleType("astropy")
    const = _t.ModuleType("astropy.constants")
    const.c = _t.SimpleNamespace(value=299792458.0)
    const.G = _t.SimpleNamespace(value=6.6743e-11)
    const.M_sun = _t.SimpleNamespace(value=1.988409870698051e30)
    astropy.constants = const
    sys.modules["astropy"] = astropy
    sys.modules["astropy.constants"] = const
    for m in [
        "llvmlite", "llvmlite.binding", "h5py", "xarray", "pandas", "seaborn",
        "matplotlib", "matplotlib.pyplot", "matplotlib.offsetbox", "sigpyproc",
        "sigpyproc.core", "sigpyproc.timeseries", "sigpyproc.viz",
        "sigpyproc.viz.styles", "rocket_fft",
    ]:
        mod = _t.ModuleType(m)
        mod.__getattr__ = lambda n: _Any()
        sys.modules[m] = mod
    orig = _md.version
    _md.version = lambda n: "0.8.0-ref" if n == "pyloki" else orig(n)
    sys.path.insert(0, reference_src)

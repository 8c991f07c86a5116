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


# Inside compiled numba code scalars have strong types (float32 * float64 is
# float64), so arguments become numpy scalars; results are boxed into Python
# scalars on return, as numba returns them.
_ARG_CASTS = {"f8": np.float64, "float64": np.float64, "f4": np.float32,
              "float32": np.float32, "i8": np.int64, "int64": np.int64, "i4": np.int32,
              "int32": np.int32, "b1": bool}
_RESULT_CASTS = {"f8": float, "float64": float, "f4": float, "float32": float, "i8": int,
                 "int64": int, "i4": int, "int32": int, "b1": bool}
_CAST_SIGNATURES = False


def _split_args(text: str) -> list[str]:
    out, depth, cur = [], 0, ""
    for ch in text:
        if ch in "[(":
            depth += 1
        elif ch in "])":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _typed(sig: str, f):
    """Cast scalar arguments and a scalar result to the types of a numba
    signature string ``ret(arg, ...)``, as compiled numba code would."""
    ret, _, rest = sig.partition("(")
    casts = [_ARG_CASTS.get(t) for t in _split_args(rest[:-1])]
    rcast = _RESULT_CASTS.get(ret.strip())

    def call(*args, **kw):
        args = [c(x) if c is not None and i < len(casts) else x
                for i, (x, c) in enumerate(zip(args, casts + [None] * len(args)))]
        r = f(*args, **kw)
        return rcast(r) if rcast is not None else r

    call.__name__ = f.__name__
    return call


def _deco(*a, **k):
    if len(a) == 1 and callable(a[0]) and not k:
        return a[0]
    sig = a[0] if a else None
    if isinstance(sig, list) and len(sig) == 1:
        sig = sig[0]
    if _CAST_SIGNATURES and isinstance(sig, str):
        return lambda f: _typed(sig, f)
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


def install(reference_src: str, cast_signatures: bool = False) -> None:
    """Install the stand-ins and put ``reference_src`` first on sys.path.
    ``cast_signatures`` makes functions with an explicit numba signature
    string cast their scalar arguments and result to its types."""
    global _CAST_SIGNATURES
    _CAST_SIGNATURES = cast_signatures
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

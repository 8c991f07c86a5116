"""CPU oracle for the FFA / scoring / pruning hot path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package; the product path (``pyloki_gb300``)
never does. ``loki_oracle.c`` restates pyloki's numba loops in C with numpy
rounding (file:line citations inside) and is pinned against fixtures that the
reference itself produced (``tests/golden``).
"""

from oracle.oracle import build, load

__all__ = ["build", "load"]

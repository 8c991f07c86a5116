"""GB300-native (sm_103a) FFA, boxcar scoring and pruning for pyloki.

Host code mirrors pyloki's API (``PulsarSearchConfig``, ``DynamicProgramming``,
``ffa_search``, ``boxcar_snr_nd``, ``Pruning``/``prune_dyp_tree``); the
arithmetic runs in hand-written CUDA kernels in ``libloki_gb300.so`` reached
through a C ABI (``include/loki_gb300.h``).
"""

from pyloki_gb300.config import C_VAL, FLOAT_EPSILON, ParamLimits, PulsarSearchConfig
from pyloki_gb300.timeseries import TimeSeries

__all__ = ["C_VAL", "FLOAT_EPSILON", "ParamLimits", "PulsarSearchConfig", "TimeSeries"]
__version__ = "0.1.0"

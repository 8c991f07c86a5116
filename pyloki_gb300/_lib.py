"""ctypes binding of ``libloki_gb300.so`` (declared in ``include/loki_gb300.h``).

The library is the product path: if it cannot be loaded the import of the
GPU entry points fails with a RuntimeError; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LOKI_OK = 0
LOKI_ERR_INVALID = -1
LOKI_ERR_CUDA = -2
LOKI_ERR_UNSUPPORTED = -3
LOKI_ERR_CAPACITY = -4

LOKI_DEVERR_WINDOW = 1
LOKI_DEVERR_BRANCH = 2
LOKI_DEVERR_TIMEOUT = 4
LOKI_DEVERR_CAPACITY = 8

MAX_PARAMS = 5
MAX_WIDTHS = 64
MAX_RESCORE_LEVELS = 24

_LIB_PATH = Path(__file__).resolve().parent / "libloki_gb300.so"


class LokiFFALevel(C.Structure):
    _fields_ = [
        ("nparams", C.c_int32),
        ("nbins", C.c_int32),
        ("level", C.c_int32),
        ("storage", C.c_int32),
        ("tseg_brute", C.c_double),
        ("counts_cur", C.c_int64 * MAX_PARAMS),
        ("counts_prev", C.c_int64 * MAX_PARAMS),
        ("limits", (C.c_double * 2) * MAX_PARAMS),
        ("param_arr", C.c_void_p * MAX_PARAMS),
        ("out_start", C.c_int64),
        ("out_width", C.c_int64),
        ("in_start", C.c_int64),
        ("in_width", C.c_int64),
        ("nseg_in", C.c_int64),
        ("last_split", C.c_void_p),
    ]


class LokiFFACoord(C.Structure):
    _fields_ = [
        ("i_tail", C.c_uint32),
        ("shift_tail", C.c_float),
        ("i_head", C.c_uint32),
        ("shift_head", C.c_float),
    ]


class LokiScoreSpec(C.Structure):
    _fields_ = [
        ("nwidths", C.c_int32),
        ("wmax", C.c_int32),
        ("mode", C.c_int32),
        ("nseg", C.c_int32),
        ("inv_stdnoise", C.c_double),
        ("widths", C.c_int32 * MAX_WIDTHS),
        ("hb", C.c_double * MAX_WIDTHS),
        ("b", C.c_double * MAX_WIDTHS),
    ]


_M6 = (C.c_double * (MAX_PARAMS + 1)) * (MAX_PARAMS + 1)


class LokiPruneLevel(C.Structure):
    _fields_ = [
        ("poly_order", C.c_int32),
        ("nbins", C.c_int32),
        ("nparams_ffa", C.c_int32),
        ("moving", C.c_int32),
        ("tiling", C.c_int32),
        ("branch_max", C.c_int32),
        ("eta_m", C.c_double),
        ("dfc", C.c_double * MAX_PARAMS),
        ("fac", C.c_double * MAX_PARAMS),
        ("tm_a", _M6),
        ("tm_i", _M6),
        ("tm_n", _M6),
        ("tm_e", _M6),
        ("dt_phase", C.c_double),
        ("n_accel", C.c_int64),
        ("n_freq", C.c_int64),
        ("accel_min", C.c_double),
        ("accel_inv", C.c_double),
        ("freq_min", C.c_double),
        ("freq_inv", C.c_double),
        ("basis", C.c_int32),
        ("reserved2", C.c_int32),
        ("tm_b", _M6),
        ("tm_be", _M6),
        ("tm_r", _M6),
        ("cfact", C.c_double * (MAX_PARAMS + 1)),
        ("ctsk", C.c_double * (MAX_PARAMS + 1)),
        ("circ_sig_prop", C.c_double),
        ("circ_sig_valid", C.c_double),
        ("circ_omega_max_sq", C.c_double),
        ("circ_x_mass", C.c_double),
        ("circ_dt_add", C.c_double),
        ("circ_dt_init", C.c_double),
        ("circ_dt_next", C.c_double),
    ]


class LokiBranchInfo(C.Structure):
    _fields_ = [
        ("first", C.c_double * MAX_PARAMS),
        ("dact", C.c_double * MAX_PARAMS),
        ("count", C.c_int32 * MAX_PARAMS),
        ("reserved", C.c_int32),
        ("d0", C.c_double),
    ]


BRANCH_INFO_BYTES = C.sizeof(LokiBranchInfo)

_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double
_PL = C.POINTER(LokiPruneLevel)

#: name -> (restype, argtypes); the exported C ABI.
class LokiPruneTree(C.Structure):
    _fields_ = [("leaves", C.c_void_p), ("folds", C.c_void_p), ("scores", C.c_void_p),
                ("scores_ep", C.c_void_p), ("backtracks", C.c_void_p), ("n", C.c_int64),
                ("cap", C.c_int64)]


class LokiPruneWork(C.Structure):
    _fields_ = [("info", C.c_void_p), ("offsets", C.c_void_p), ("scan", C.c_void_p),
                ("scan_bytes", C.c_int64), ("par_cap", C.c_int64),
                ("child_scores", C.c_void_p), ("child_idx", C.c_void_p),
                ("child_phase", C.c_void_p), ("surv", C.c_void_p), ("sscan", C.c_void_p),
                ("sscan_bytes", C.c_int64), ("child_cap", C.c_int64), ("n_surv", C.c_void_p),
                ("minmax", C.c_void_p), ("ovf_ids", C.c_void_p), ("ovf_keys", C.c_void_p),
                ("ovf_thr", C.c_void_p), ("ovf_cap", C.c_int64), ("host_words", C.c_void_p),
                ("ev_score_begin", C.c_void_p), ("ev_score_end", C.c_void_p)]


class LokiPruneLevelResult(C.Structure):
    _fields_ = [("n_parents", C.c_int64), ("n_children", C.c_int64), ("n_surv", C.c_int64),
                ("score_min", C.c_float), ("score_max", C.c_float), ("overflow", C.c_int32),
                ("dev_err", C.c_int32), ("need_par_cap", C.c_int64),
                ("need_child_cap", C.c_int64), ("need_ovf_cap", C.c_int64),
                ("need_tree_cap", C.c_int64)]


class LokiPruneLevelStats(C.Structure):
    _fields_ = [("n_parents", C.c_int64), ("n_children", C.c_int64), ("n_valid", C.c_int64),
                ("n_surv", C.c_int64), ("score_min", C.c_float), ("score_max", C.c_float),
                ("overflow", C.c_int32), ("reserved", C.c_int32)]


class LokiPruneRun(C.Structure):
    _fields_ = [("trees", LokiPruneTree * 2), ("work", LokiPruneWork), ("counts", C.c_void_p),
                ("ovf_flag", C.c_void_p), ("stats", C.c_void_p), ("best_leaves", C.c_void_p),
                ("best_scores", C.c_void_p), ("bt_hist", C.c_void_p), ("bt_rows", C.c_int64),
                ("exp_off", C.c_void_p), ("child_map", C.c_void_p), ("valid_flags", C.c_void_p),
                ("valid_ids", C.c_void_p), ("child_class", C.c_void_p),
                ("batch_taylor", C.c_void_p), ("batch_offsets", C.c_void_p)]


class LokiPruneJob(C.Structure):
    _fields_ = [("ffa_fold", C.c_void_p), ("seg_stride", C.c_int64), ("seed_n", C.c_int64),
                ("run", LokiPruneRun), ("dev_err", C.c_void_p)]


class LokiSeedJob(C.Structure):
    _fields_ = [("seed_leaves", C.c_void_p), ("fold_rows", C.c_void_p), ("n", C.c_int64),
                ("leaves_out", C.c_void_p), ("folds_out", C.c_void_p),
                ("scores_out", C.c_void_p), ("scores_ep_out", C.c_void_p),
                ("seed_scores_out", C.c_void_p), ("bt_out", C.c_void_p),
                ("dev_err", C.c_void_p)]


class LokiAscendJob(C.Structure):
    _fields_ = [("lvl", LokiPruneLevel), ("leaves", C.c_void_p), ("folds", C.c_void_p),
                ("scores", C.c_void_p), ("scores_ep", C.c_void_p), ("n_dev", C.c_void_p),
                ("tm_seg", C.c_void_p), ("dt_seg", C.c_void_p), ("seg_idx", C.c_void_p),
                ("ffa_fold", C.c_void_p), ("seg_stride", C.c_int64), ("dev_err", C.c_void_p)]


class LokiGatherPart(C.Structure):
    _fields_ = [("src", C.c_void_p), ("bytes", C.c_int64), ("dst_off", C.c_int64)]


#: numpy view of an array of LokiPruneLevelStats records
PRUNE_STATS_DTYPE = np.dtype([("n_parents", np.int64), ("n_children", np.int64),
                              ("n_valid", np.int64), ("n_surv", np.int64),
                              ("score_min", np.float32), ("score_max", np.float32),
                              ("overflow", np.int32), ("reserved", np.int32)])


class LokiMLP(C.Structure):
    _fields_ = [("w1", C.c_void_p), ("b1", C.c_void_p), ("w2", C.c_void_p),
                ("b2", C.c_void_p), ("w3", C.c_void_p), ("b3", C.c_void_p)]


class LokiMLPGrad(C.Structure):
    _fields_ = [("w1", C.c_void_p), ("b1", C.c_void_p), ("w2", C.c_void_p),
                ("b2", C.c_void_p), ("w3", C.c_void_p), ("b3", C.c_void_p),
                ("loss", C.c_void_p)]


MOD_MAX_COEFFS = 16
PULSE_MAX_NBINS = 12288
MOD_KINDS = {"derivative": 0, "derivative_series": 1, "circular": 2, "circular_t0": 3,
             "keplerian": 4, "table": 5}


class LokiModulation(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ncoeff", C.c_int32), ("t_ref", C.c_double),
                ("c", C.c_double * MOD_MAX_COEFFS)]


class LokiPulseSpec(C.Structure):
    _fields_ = [("dt", C.c_double), ("period", C.c_double), ("snr", C.c_double),
                ("ducy", C.c_double), ("phi0", C.c_double), ("nbins", C.c_int32),
                ("ngrid", C.c_int32), ("lut_off", C.c_int64), ("seed", C.c_uint64),
                ("mod", LokiModulation)]


SIGNATURES: dict[str, tuple] = {
    "loki_version": (C.c_int, []),
    "loki_last_error": (C.c_char_p, []),
    "loki_launch_count": (C.c_int64, []),
    "loki_brutefold": (C.c_int, [_P, _P, _I64, _P, _I64, _I64, _I32, _D, _D, _P, _I64, _P, _P]),
    "loki_brutefold_unit_variance": (C.c_int, [_P, _I64, _P, _I64, _I64, _I32, _D, _D, _P,
                                                _I64, _P, _P]),
    "loki_brutefold_noalloc": (C.c_int, [_P, _P, _I64, _P, _I64, _I64, _I32, _D, _D, _P, _P]),
    "loki_brutefold_noalloc_scratch_bytes": (C.c_int64, []),
    "loki_brutefold_scratch_bytes": (C.c_int64, [_I64, _I64, _I32]),
    "loki_prune_run_blocks": (C.c_int, [_P, _I32, _P, _P, _P, _I32, C.POINTER(LokiScoreSpec),
                                        _I64, _I64, _P, _I64, _P]),
    "loki_prune_run_blocks_scratch_bytes": (C.c_int64, [_I32, _I32]),
    "loki_prune_run_batch": (C.c_int, [_P, _I32, _P, _P, _P, _I32, C.POINTER(LokiScoreSpec),
                                       _I64, _I64, _P, _I64, _P]),
    "loki_prune_batch_tables": (C.c_int, [_P, _I32, _P, _P, _P, _I32,
                                          C.POINTER(LokiScoreSpec), _I64, _I64, _I32, _P, _I64,
                                          _P, _P]),
    "loki_prune_batch_enqueue": (C.c_int, [_P, _I32, _I32, C.POINTER(LokiScoreSpec), _I64,
                                           _I64, _P, _P]),
    "loki_prune_batch_score_times": (C.c_int, [_P, _I32, _I32, C.POINTER(LokiScoreSpec),
                                               _I64, _I64, _P, _P, _P]),
    "loki_prune_ascend_batch": (C.c_int, [_P, _I32, _I32, C.POINTER(LokiScoreSpec), _I64,
                                          _I32, _P, _I64, _P]),
    "loki_gather_parts": (C.c_int, [_P, _I32, _P, _I64, _P, _I64, _P]),
    "loki_prune_seed_batch": (C.c_int, [_P, _I32, _I32, _I32, C.POINTER(LokiScoreSpec), _P,
                                        _I64, _P]),
    "loki_ffa_plan": (C.c_int, [C.POINTER(LokiFFALevel), _P, _P, _P]),
    "loki_ffa_level": (C.c_int, [C.POINTER(LokiFFALevel), _P, _P, _P, _P]),
    "loki_ffa_level_score": (C.c_int, [C.POINTER(LokiFFALevel), _P, C.POINTER(LokiScoreSpec),
                                       _P, _P, _P]),
    "loki_ffa_band_windows": (C.c_int, [C.POINTER(LokiFFALevel), _I64, _P, _P, _P]),
    "loki_ffa_final_banded": (C.c_int, [C.POINTER(LokiFFALevel), C.POINTER(LokiFFALevel), _I64,
                                        _P, _P, _P, _P, _I64, C.POINTER(LokiScoreSpec), _P, _P,
                                        _P]),
    "loki_ffa_final_banded_scratch": (C.c_int64, [C.POINTER(LokiFFALevel),
                                                  C.POINTER(LokiFFALevel), _I64]),
    "loki_ffa_final_tiled": (C.c_int, [C.POINTER(LokiFFALevel), C.POINTER(LokiFFALevel), _P,
                                       _P, _I64, C.POINTER(LokiScoreSpec), _I32, _P, _P, _P]),
    "loki_ffa_final_tiled_scratch": (C.c_int64, [C.POINTER(LokiFFALevel),
                                                 C.POINTER(LokiFFALevel)]),
    "loki_boxcar_snr": (C.c_int, [_P, _I64, _I32, C.POINTER(LokiScoreSpec), _P, _P]),
    "loki_snr_score_batch": (C.c_int, [_P, _I64, _I32, C.POINTER(LokiScoreSpec), _P, _P]),
    "loki_fold_norm": (C.c_int, [_P, _I64, _I32, _P, _P]),
    "loki_f32_to_bf16": (C.c_int, [_P, _I64, _P, _P]),
    "loki_sim_score_folds": (C.c_int, [_P, _P, _P, _I64, _P, _I32, C.c_float, C.c_float,
                                       C.c_uint64, C.POINTER(LokiScoreSpec), _P, _P, _P]),
    "loki_gather_rows": (C.c_int, [_P, _P, _I64, _I64, _P, _P]),
    "loki_pulse_template": (C.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _P]),
    "loki_pulse_fold": (C.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _I32, _P, _P, _P]),
    "loki_pulse_apply": (C.c_int, [_P, _I32, _I64, _P, _P, _P]),
    "loki_fold_ephem": (C.c_int, [_P, _P, _I64, _D, C.POINTER(LokiModulation), _P, _D, _I32,
                                  _I32, _P, _P, _P, _P]),
    "loki_downsample": (C.c_int, [_P, _I64, _I32, _P, _P]),
    "loki_running_median": (C.c_int, [_P, _I64, _I32, _I32, _P, _P]),
    "loki_select_kth": (C.c_int, [_P, _I64, _I64, _P, _P, _I64, _P]),
    "loki_select_scratch_bytes": (C.c_int64, []),
    "loki_sum_f64": (C.c_int, [_P, _I64, _I32, _P, _P, _I64, _P]),
    "loki_affine": (C.c_int, [_P, _I64, C.c_float, C.c_float, _P, _P]),
    "loki_kadane_circular": (C.c_int, [_P, _I64, _I32, _P, _I32, _P, _P, _P, _P]),
    "loki_matched_filter": (C.c_int, [_P, _I64, _I32, _P, _I32, _I32, C.c_float, _P, _P, _P]),
    "loki_matched_filter_conv": (C.c_int, [_P, _I64, _I32, _P, _I32, _P, _P]),
    "loki_matched_filter_double": (C.c_int, [_P, _I64, _I32, _P, _I32, _P, _I32, _P, _I32, _D,
                                             _D, _P, _I32, _D, _D, _P, _P]),
    "loki_harmonic_sum": (C.c_int, [_P, _I64, _I32, _I32, _P, _I32, _I32, _D, _D, _P, _I32,
                                    _D, _D, _P, _P]),
    "loki_pulse_calibrate": (C.c_int, [_P, _I32, _P, _I32, _I32, _D, _P, _P]),
    "loki_pulse_emit": (C.c_int, [_P, _I32, _I64, _P, _P, _P, _P, _P, _P, _P]),
    "loki_mlp_smem_bytes": (C.c_int64, []),
    "loki_branch_features": (C.c_int, [_P, _P, _I64, _I32, C.c_float, C.c_float, C.c_float,
                                       C.c_float, _P, _P, _P]),
    "loki_mlp_force_timeout": (C.c_int, [_I32]),
    "loki_mlp_forward": (C.c_int, [C.POINTER(LokiMLP), _P, _I64, _P, _P, _P]),
    "loki_mlp_backward": (C.c_int, [C.POINTER(LokiMLP), _P, _P, _P, _I64, C.c_float,
                                    C.POINTER(LokiMLPGrad), _P, _P, _P]),
    "loki_mlp_adam": (C.c_int, [_P, _P, _P, _P, _I64, C.c_float, C.c_float, C.c_float,
                                C.c_float, _I64, _P]),
    "loki_ffa_rescore": (C.c_int, [C.POINTER(LokiFFALevel), _I32, _P, _P, _I64, _D, _I64, _P,
                                   _I64, _P, _P, _I64, _I64, C.POINTER(LokiScoreSpec), _P, _P,
                                   _P]),
    "loki_brutefold_complex": (C.c_int, [_P, _P, _I64, _P, _I64, _I64, _I32, _D, _D, _P, _P]),
    "loki_ffa_level_complex": (C.c_int, [C.POINTER(LokiFFALevel), _P, _P, _P, _P]),
    "loki_fold_norm_complex": (C.c_int, [_P, _I64, _I32, _P, _P]),
    "loki_scan_scratch_bytes": (C.c_int64, [_I64]),
    "loki_prune_branch": (C.c_int, [_PL, _P, _I64, _P, _P, _P, _I64, _P, _P]),
    "loki_prune_branch_masked": (C.c_int, [_PL, _P, _I64, _P, _P, _P, _P, _I64, _P, _P]),
    "loki_prune_best": (C.c_int, [_P, _I64, _P, _I32, _P, _P, _P]),
    "loki_prune_ascend_dev": (C.c_int, [_PL, _P, _P, _P, _P, _P, _I64, _I32, _P, _P, _P, _P,
                                        _I64, C.POINTER(LokiScoreSpec), _P, _P]),
    "loki_prune_run": (C.c_int, [_PL, _I32, _P, _I64, _P, _P, C.POINTER(LokiScoreSpec), _I64,
                                 _I64, _I64, C.POINTER(LokiPruneRun), _P, _P]),
    "loki_prune_level": (C.c_int, [_PL, C.POINTER(LokiPruneTree), C.POINTER(LokiPruneTree),
                                   C.POINTER(LokiPruneWork), _P, C.POINTER(LokiScoreSpec), _D,
                                   _I64, _I64, _P, C.POINTER(LokiPruneLevelResult), _P, _P]),
    "loki_prune_score": (C.c_int, [_PL, _P, _P, _I64, _P, _P, _I64, _P,
                                   C.POINTER(LokiScoreSpec), _P, _P, _P, _P, _P, _P]),
    "loki_prune_select": (C.c_int, [_P, _I64, _D, _P, _P, _P, _I64, _P]),
    "loki_prune_select_overflow": (C.c_int, [_P, _P, _I64, _I64, _D, _I64, _P, _P, _P, _P,
                                             _P, _I64, _P]),
    "loki_prune_emit": (C.c_int, [_PL, _P, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P,
                                  _P, _P, _P, _P, _P]),
    "loki_prune_ascend": (C.c_int, [_PL, _P, _P, _P, _P, _I64, _I32, _P, _P, _P, _P, _I64,
                                    C.POINTER(LokiScoreSpec), _P, _P]),
    "loki_prune_score_complex": (C.c_int, [_PL, _P, _P, _I64, _P, _P, _I64, _P,
                                           C.POINTER(LokiScoreSpec), _P, _P, _P, _P, _P, _P]),
    "loki_prune_emit_complex": (C.c_int, [_PL, _P, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P,
                                          _P, _P, _P, _P, _P, _P]),
    "loki_prune_ascend_complex": (C.c_int, [_PL, _P, _P, _P, _P, _I64, _I32, _P, _P, _P, _P,
                                            _I64, C.POINTER(LokiScoreSpec), _P, _P]),
    "loki_prune_circ_branch": (C.c_int, [_PL, _P, _I64, _P, _P, _P, _P, _I64, _P, _P]),
    "loki_prune_circ_map": (C.c_int, [_PL, _P, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "loki_prune_circ_score": (C.c_int, [_PL, _P, _P, _I64, _I64, _P, _P, _P, _P, _P, _I64, _P,
                                        C.POINTER(LokiScoreSpec), _P, _P, _P, _P, _P, _P, _P,
                                        _P, _P]),
    "loki_prune_circ_emit": (C.c_int, [_PL, _P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P,
                                       _P, _P, _P, _P, _P, _P, _P, _P]),
    "loki_prune_circ_score_complex": (C.c_int, [_PL, _P, _P, _I64, _I64, _P, _P, _P, _P, _P,
                                                _I64, _P, C.POINTER(LokiScoreSpec), _P, _P, _P,
                                                _P, _P, _P, _P, _P, _P]),
    "loki_prune_circ_emit_complex": (C.c_int, [_PL, _P, _P, _I64, _P, _P, _P, _P, _P, _I64, _P,
                                               _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
}

#: bytes of one circular-tree child record (parent, cartesian index, crackle index, pad)
CIRC_CHILD_BYTES = 16

_lock = threading.Lock()
_lib: C.CDLL | None = None


def lib_path() -> Path:
    return _LIB_PATH


def load(path: str | Path | None = None) -> C.CDLL:
    """Load the library (once) and bind the C ABI prototypes."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path is not None else _LIB_PATH
        if not p.exists():
            msg = (f"{p} is missing: build it with `python -m pyloki_gb300.build` "
                   "(the GPU path has no CPU fallback)")
            raise RuntimeError(msg)
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


class LokiError(RuntimeError):
    """A CUDA-side failure reported by libloki_gb300."""


def check(rc: int) -> None:
    """Map a status code to the reference's exception types."""
    if rc == LOKI_OK:
        return
    msg = load().loki_last_error().decode(errors="replace")
    if rc in (LOKI_ERR_INVALID, LOKI_ERR_CAPACITY):
        raise ValueError(msg)
    if rc == LOKI_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise LokiError(msg)


def check_dev_err(err_word) -> None:
    """Raise if a kernel reported a device-side range error (syncs the stream)."""
    v = int(err_word.item())
    if v & LOKI_DEVERR_WINDOW:
        msg = "resolved grid index fell outside the input frequency window"
        raise LokiError(msg)
    if v & LOKI_DEVERR_BRANCH:
        msg = "Invalid input: increase branch_max."
        raise ValueError(msg)
    if v & LOKI_DEVERR_TIMEOUT:
        msg = "a bounded wait for the tensor cores timed out"
        raise LokiError(msg)
    if v & LOKI_DEVERR_CAPACITY:
        msg = "a device-counted run outgrew its workspace"
        raise LokiError(msg)
    if v:
        msg = f"device error word {v}"
        raise LokiError(msg)


def ptr(t) -> int:
    """Device pointer of a torch tensor (or 0 for None)."""
    return 0 if t is None else int(t.data_ptr())


def stream_ptr(stream) -> int:
    return int(stream.cuda_stream) if stream is not None else 0


def score_spec(widths, nbins: int, stdnoise: float = 1.0, mode: int = 0) -> LokiScoreSpec:
    """Boxcar constants with the reference's float64 expressions
    (``detection/scoring.py:127-138``): h = sqrt((n-w)/(n*w)), b = w*h/(n-w)."""
    widths = np.asarray(widths, dtype=np.int64)
    if widths.ndim != 1 or not 1 <= len(widths) <= MAX_WIDTHS:
        msg = f"need 1..{MAX_WIDTHS} boxcar widths, got {widths.shape}"
        raise ValueError(msg)
    sp = LokiScoreSpec()
    sp.nwidths = len(widths)
    sp.wmax = int(widths.max())
    sp.mode = mode
    sp.inv_stdnoise = 1.0 / stdnoise
    size = np.int64(nbins)
    for i, width in enumerate(widths):
        size_w = size - width
        height = np.sqrt(size_w / (size * width))
        b = width * height / size_w
        sp.widths[i] = int(width)
        sp.hb[i] = float(height + b)
        sp.b[i] = float(b)
    return sp

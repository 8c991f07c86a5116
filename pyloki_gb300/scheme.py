"""Middle-out segment order and reference coordinates (``utils/snail.py:18-389``).

Host-side plan of an enumerate-prune run: which FFA segment is added at each
level and the (t0, scale) coordinates the pruning level uses. Pure FP64
scalar arithmetic with the reference's operation order.
"""

from __future__ import annotations

import numpy as np


class MiddleOutScheme:
    """Segments ordered by distance from ``ref_idx`` (ties: lower index first)."""

    def __init__(self, nsegments: int, ref_idx: int, tsegment: float, stride: int = 1) -> None:
        if nsegments <= 0:
            msg = f"nsegments must be greater than 0, got {nsegments}."
            raise ValueError(msg)
        if ref_idx < 0 or ref_idx >= nsegments:
            msg = f"ref_idx must be in [0, {nsegments}), got {ref_idx}."
            raise ValueError(msg)
        if tsegment <= 0:
            msg = f"tsegment must be greater than 0, got {tsegment}."
            raise ValueError(msg)
        if stride <= 0:
            msg = f"stride must be greater than 0, got {stride}."
            raise ValueError(msg)
        self.nsegments = nsegments
        self.ref_idx = ref_idx
        self.tsegment = tsegment
        self.stride = stride
        self.data = np.argsort(np.abs(np.arange(nsegments) - ref_idx), kind="mergesort")

    def _check(self, level: int) -> None:
        if level < 0 or level >= self.nsegments:
            msg = f"level must be in [0, {self.nsegments - 1}], got {level}."
            raise ValueError(msg)

    def get_segment_idx(self, level: int) -> int:
        self._check(level)
        return int(self.data[level])

    def get_coord(self, level: int) -> tuple[float, float]:
        self._check(level)
        till = self.data[: level + 1]
        ref = (np.min(till) + np.max(till) + 1) / 2
        scale = ref - np.min(till)
        return float(ref * self.tsegment), float(scale * self.tsegment)

    def get_segment_coord(self, level: int) -> tuple[float, float]:
        self._check(level)
        ref = (self.get_segment_idx(level) + 0.5) * self.tsegment
        return ref, 0.5 * self.tsegment

    def get_segment_coords_so_far(self, level: int) -> tuple[np.ndarray, np.ndarray]:
        self._check(level)
        res = np.zeros((level + 1, 2), dtype=np.float64)
        seg_idx = np.zeros(level + 1, dtype=np.int64)
        for i in range(level + 1):
            res[i, 0] = (self.get_segment_idx(i) + 0.5) * self.tsegment
            res[i, 1] = 0.5 * self.tsegment
            seg_idx[i] = self.get_segment_idx(i)
        return seg_idx, res

    def _fixed(self, level: int, t0_out: str) -> tuple[float, float]:
        t0_init, scale_init = self.get_coord(0)
        t0_next, scale_next = self.get_coord(level)
        left_edge = t0_next - scale_next
        right_edge = t0_next + scale_next
        scale_cur = max(abs(left_edge - t0_init), abs(right_edge - t0_init))
        return (t0_init if t0_out == "init" else t0_next), scale_cur - scale_init

    def get_current_coord(self, level: int, moving_grid: bool) -> tuple[float, float]:
        self._check(level)
        if level == 0:
            return self.get_coord(level)
        if moving_grid:
            prev_ref, _ = self.get_coord(level - 1)
            _, cur_scale = self.get_coord(level)
            return prev_ref, cur_scale
        return self._fixed(level, "init")

    def get_previous_coord(self, level: int, moving_grid: bool) -> tuple[float, float]:
        level = level - 1
        self._check(level)
        if level == 0 or moving_grid:
            return self.get_coord(level)
        return self._fixed(level, "init")

    def get_report_coord(self, moving_grid: bool) -> tuple[float, float]:
        level = self.nsegments - 1
        if moving_grid:
            return self.get_coord(level)
        return self._fixed(level, "next")


def determine_ref_segs_pareto(nsegments: int, n_runs: int) -> list[int]:
    """Pareto-spaced reference segments (``utils/np_utils.py:412-443``)."""
    if not (1 <= n_runs <= nsegments):
        msg = f"n_runs must be between 1 and {nsegments}"
        raise ValueError(msg)
    if n_runs == 1:
        return [nsegments // 2]

    def round_div(num: int, den: int) -> int:
        return (num + den // 2) // den

    margin = round_div(nsegments - 1, 2 * n_runs)
    lo = margin
    hi = nsegments - 1 - margin
    denom = n_runs - 1
    return [round_div((denom - i) * lo + i * hi, denom) for i in range(n_runs)]

"""Pruning result files (``io/cands.py:106-411``): the reference's HDF5
layout, written and read through ``pyloki_gb300.h5``.

A result file holds, as the reference writes it with h5py:

- file attributes ``pruning_version`` (str), ``param_names`` (str array),
  ``nsegments`` and ``max_sugg`` (int64), and the dataset
  ``threshold_scheme``;
- per run, group ``runs/<ref_seg:03d>_<task:02d>`` with datasets ``scheme``,
  ``param_sets``, ``scores_ep``, ``scores``, ``level_stats`` (compound, one
  row per level) and ``timer_stats`` (compound, one row).

The reference compresses every dataset with gzip; this writer stores them
uncompressed (contiguous), which every HDF5 reader reads the same way.
"""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np

from pyloki_gb300 import h5

#: per-step timers of a run (io/cands.py:111-120)
TIMER_NAMES = ["branch", "validate", "resolve", "shift_add", "score", "threshold",
               "transform", "batch_add"]

#: one row of ``level_stats`` (io/cands.py:199-211)
LEVEL_DTYPE = np.dtype([("level", np.int32), ("seg_idx", np.int32), ("threshold", np.float32),
                        ("score_min", np.float32), ("score_max", np.float32),
                        ("n_branches", np.int32), ("n_leaves", np.int32),
                        ("n_leaves_phy", np.int32), ("n_leaves_surv", np.int32)])
TIMER_DTYPE = np.dtype([(name, np.float32) for name in TIMER_NAMES])


class PruneStatsCollection:
    """Level statistics and step timers of one run (``io/cands.py:106-274``)."""

    TIMER_NAMES = TIMER_NAMES

    def __init__(self, stats_list=None, timers: dict | None = None) -> None:
        self.stats_list = list(stats_list or [])
        self.timers = dict.fromkeys(TIMER_NAMES, 0.0)
        if timers:
            self.timers.update({k: float(v) for k, v in timers.items()})

    @property
    def nstages(self) -> int:
        return len(self.stats_list)

    def update_stats(self, stats) -> None:
        self.stats_list.append(stats)

    def update_timers(self, timers: dict) -> None:
        for k, v in timers.items():
            self.timers[k] = self.timers.get(k, 0.0) + float(v)

    def to_array(self) -> tuple[np.ndarray, np.ndarray]:
        """``level_stats`` and ``timer_stats`` records (io/cands.py:197-227)."""
        level_stats = np.zeros(len(self.stats_list), dtype=LEVEL_DTYPE)
        for i, s in enumerate(self.stats_list):
            level_stats[i] = (s.level, s.seg_idx, s.threshold, s.score_min, s.score_max,
                              s.n_branches, s.n_leaves, s.n_leaves_phy, s.n_leaves_surv)
        timer_stats = np.zeros(1, dtype=TIMER_DTYPE)
        for name in TIMER_NAMES:
            timer_stats[0][name] = self.timers.get(name, 0.0)
        return level_stats, timer_stats

    @classmethod
    def from_arrays(cls, level_stats: np.ndarray, timer_stats: np.ndarray
                    ) -> PruneStatsCollection:
        """Inverse of ``to_array`` (io/cands.py:240-274)."""
        from pyloki_gb300.prune import PruneStats

        col = cls()
        for row in level_stats:
            col.update_stats(PruneStats(
                level=int(row["level"]), seg_idx=int(row["seg_idx"]),
                threshold=float(row["threshold"]), score_min=float(row["score_min"]),
                score_max=float(row["score_max"]), n_branches=int(row["n_branches"]),
                n_leaves=int(row["n_leaves"]), n_leaves_phy=int(row["n_leaves_phy"]),
                n_leaves_surv=int(row["n_leaves_surv"])))
        for name in TIMER_NAMES:
            col.timers[name] = float(timer_stats[0][name])
        return col


class PruneResultWriter:
    """``io/cands.py:277-355``: a context manager over one result file
    (mode "w" creates it, "a" adds runs to it)."""

    def __init__(self, filename, mode: str = "w") -> None:
        self.filename = Path(filename)
        self.mode = mode
        self.file: h5.File | None = None
        self.runs_group: h5.Group | None = None

    def __enter__(self) -> PruneResultWriter:
        self.file = h5.File(self.filename, self.mode)
        self.runs_group = self.file.require_group("runs")
        return self

    def __exit__(self, exc_type, exc_val, exc_tb) -> None:
        if self.file is not None:
            self.file.close()
            self.file = None

    def write_metadata(self, param_names, nsegments: int, max_sugg: int,
                       threshold_scheme) -> None:
        if self.file is None:
            msg = "File not open."
            raise ValueError(msg)
        from pyloki_gb300 import __version__

        self.file.attrs["pruning_version"] = __version__
        self.file.attrs["param_names"] = [str(p) for p in param_names]
        self.file.attrs["nsegments"] = np.int64(nsegments)
        self.file.attrs["max_sugg"] = np.int64(max_sugg)
        # a second call fails as h5py's create_dataset does: the name exists
        self.file.create_dataset("threshold_scheme", data=np.asarray(threshold_scheme))

    def write_run_results(self, run_name: str, scheme, leaves_report, scores, scores_ep,
                          pstats) -> None:
        """One run's group; ``pstats`` is a ``PruneStatsCollection`` or a
        list of ``PruneStats``."""
        if self.runs_group is None:
            msg = "No runs group found in the file."
            raise ValueError(msg)
        if run_name in self.runs_group:
            msg = f"Run name {run_name} already exists in the file."
            raise ValueError(msg)
        if not isinstance(pstats, PruneStatsCollection):
            pstats = PruneStatsCollection(pstats)
        level_stats, timer_stats = pstats.to_array()
        g = self.runs_group.create_group(run_name)
        for name, data in (("scheme", scheme), ("param_sets", leaves_report),
                           ("scores_ep", scores_ep), ("scores", scores),
                           ("level_stats", level_stats), ("timer_stats", timer_stats)):
            g.create_dataset(name, data=np.asarray(data))


def extract_ref_seg(file_path: Path) -> int:
    """The reference segment of a temporary run file (io/cands.py:358-363)."""
    match = re.search(r"tmp_(\d{3})_\d{2}_(log\.txt|results\.h5)", Path(file_path).name)
    return int(match.group(1)) if match else 0


def merge_prune_result_files(results_dir, log_file: Path, result_file: Path) -> None:
    """Append the temporary per-run logs and result files of ``results_dir``
    to ``log_file`` and ``result_file`` in reference-segment order, skipping
    runs already present, and delete them (io/cands.py:365-411)."""
    results_dir = Path(results_dir)
    temp_logs = sorted(results_dir.glob("tmp_*_log.txt"), key=extract_ref_seg)
    temp_h5 = sorted(results_dir.glob("tmp_*_results.h5"), key=extract_ref_seg)
    with Path(log_file).open("a") as main_log:
        for p in temp_logs:
            main_log.write(p.read_text())
            p.unlink()
    with h5.File(result_file, "a") as main:
        runs = main.require_group("runs")
        for p in temp_h5:
            tmp = h5.read_file(p)
            if "runs" in tmp:
                for run_name in tmp["runs"]:
                    if run_name in runs:
                        continue
                    tmp.copy(f"runs/{run_name}", runs)
            p.unlink()


def read_prune_results(path) -> dict:
    """A result file as plain values: ``{"attrs": {...}, "threshold_scheme":
    array, "runs": {name: {dataset: array}}}``."""
    f = h5.read_file(path)
    out = {"attrs": dict(f.attrs),
           "threshold_scheme": f["threshold_scheme"].data if "threshold_scheme" in f else None,
           "runs": {}}
    if "runs" in f:
        for name in f["runs"]:
            g = f["runs"][name]
            out["runs"][name] = {k: g[k].data for k in g}
    return out


__all__ = ["LEVEL_DTYPE", "TIMER_DTYPE", "TIMER_NAMES", "PruneResultWriter",
           "PruneStatsCollection", "extract_ref_seg", "merge_prune_result_files",
           "read_prune_results"]

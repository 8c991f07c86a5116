"""Design the per-level pruning thresholds of the circular-orbit benchmark search.

The search is the Taylor tree to the 4th derivative over 2^22 samples at
64 us, 128 segments, reference segment 64 (``bench.make_prune_cfg``). Its
thresholds come from the reference's design workflow
(``examples/optimal_thresholds.ipynb``):

1. the branching pattern of the tree (``generate_branching_pattern``,
   ``config.py:758-819``; here ``pyloki_gb300.branching``, pinned bit-exact
   to the reference by ``tests/test_branching.py``);
2. ``DynamicThresholdScheme`` (``detection/thresholding.py:702-1008``) with
   the notebook's design parameters (100 thresholds, 30 probability bins,
   1024 trials, beam 2.5, improved mode, 11 neighbours), for the injected
   pulse of the benchmark (duty cycle 0.05, S/N 10) scored at the search's
   own boxcar widths;
3. the least-cost path keeping at least 90 % of the injected signals
   (``DynamicThresholdSchemeAnalyser.backtrack_best(min_probs=[0.9])``),
   rounded to one decimal as the notebook does before pruning.

Needs a GPU (the Monte-Carlo folds run on it); the result is committed as
``prune_scheme_taylor4.npz`` and read by the benchmark and the full-size
pruning test. ``python tests/golden/make_prune_scheme.py [OUT_DIR]`` (default:
this folder).
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

REF_SEG = 64
DESIGN = {"ref_ducy": 0.05, "nbins": 64, "ntrials": 1024, "nprobs": 30, "prob_min": 0.05,
          "snr_final": 10.0, "nthresholds": 100, "beam_width": 2.5, "mode": "improved",
          "seed": 1}
MIN_PROB = 0.9
ALT_PROBS = [0.1, 0.3, 0.5, 0.7, 0.9]  # paths kept beside the chosen one
THRES_NEIGH = 11


def main() -> None:
    import torch

    import bench
    from pyloki_gb300.branching import generate_branching_pattern
    from pyloki_gb300.thresholds import DynamicThresholdScheme

    cfg = bench.make_prune_cfg()
    bp = generate_branching_pattern(cfg, "poly_taylor_moving", ref_seg=REF_SEG)
    ds = DynamicThresholdScheme(bp, DESIGN["ref_ducy"], DESIGN["nbins"],
                                ntrials=DESIGN["ntrials"], nprobs=DESIGN["nprobs"],
                                prob_min=DESIGN["prob_min"], snr_final=DESIGN["snr_final"],
                                nthresholds=DESIGN["nthresholds"], ducy_max=cfg.ducy_max,
                                wtsp=cfg.wtsp, beam_width=DESIGN["beam_width"],
                                mode=DESIGN["mode"], seed=DESIGN["seed"],
                                device=torch.device("cuda", 0))
    ds.run(thres_neigh=THRES_NEIGH)
    paths = ds.backtrack_best(ALT_PROBS)
    extra = {}
    for p, path in zip(ALT_PROBS, paths):
        if len(path) == len(bp):
            extra[f"thresholds_p{round(100 * p):02d}"] = np.around(path["threshold"], 1)
            extra[f"path_p{round(100 * p):02d}"] = path
        print({"min_prob": p, "stages": len(path),
               "success_h1_cumul": float(path["success_h1_cumul"][-1]) if len(path) else None,
               "complexity_cumul": float(path["complexity_cumul"][-1]) if len(path) else None,
               "first": np.around(path["threshold"][:6], 1).tolist() if len(path) else None,
               "last": np.around(path["threshold"][-3:], 1).tolist() if len(path) else None})
    key = f"thresholds_p{round(100 * MIN_PROB):02d}"
    if key not in extra:
        sys.exit(f"no complete scheme keeps {MIN_PROB} of the signals")
    out_dir = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE
    np.savez_compressed(out_dir / "prune_scheme_taylor4.npz", thresholds=extra[key],
                        branching_pattern=bp, ref_seg=np.int64(REF_SEG),
                        min_prob=np.float64(MIN_PROB), ducy_max=np.float64(cfg.ducy_max),
                        wtsp=np.float64(cfg.wtsp), alt_probs=np.asarray(ALT_PROBS), **extra,
                        **{k: np.asarray(v) for k, v in DESIGN.items()})


if __name__ == "__main__":
    main()

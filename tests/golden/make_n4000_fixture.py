#!/usr/bin/env python3
"""Final-state fixture of BRUSS2D-MIX at N=4000 (n = 32,000,000), DOPRI5(4),
tol 1e-6, alpha 2e-3, t in [0, 0.5]: the mixed-precision configuration's FP64
ground truth.

The reference's own solver needs hours for this size on a CPU, so the fixture
comes from the exact FP64 GPU form, which reproduces the reference bit for bit
wherever the two have been compared (every golden case up to N=2000, including
the full N=2000 DOPRI5(4) and DOPRI8(7) runs: same step counts, same final
state).  Recorded:

  steps / accepted / rejected, y_sha256, y_first/last/min/max (as the other
      golden fixtures)
  sample  -- <name>_sample.npy: the final state at the component indices of
             sample_indices() below (the first and last grid rows in full, and
             every 977th component, which alternates u and v)
  mixed   -- the mixed form's result of the same solve, measured once against
             the whole FP64 state: its step counts and relative max-norm error

Needs a GPU; run as
    python tests/golden/make_n4000_fixture.py --out <dir>
and copy the two files into tests/golden/.
"""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

NAME = "bruss_n4000_dopri54_tol1e-6"
GRID_N, ALPHA, TOL, T0, TE = 4000, 2e-3, 1e-6, 0.0, 0.5
SAMPLE_STRIDE = 977


def sample_indices(grid_n=GRID_N):
    """Indices of the stored components: grid rows 0 and N-1 (u and v of every
    column) and every SAMPLE_STRIDE-th component, sorted, without repeats."""
    row = 2 * grid_n
    n = row * grid_n
    idx = np.concatenate([np.arange(row), np.arange(n - row, n), np.arange(0, n, SAMPLE_STRIDE)])
    return np.unique(idx)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    import rk_gb300 as rk

    os.makedirs(a.out, exist_ok=True)
    prob = rk.bruss2d_mix(GRID_N, ALPHA)
    y0 = rk.ode_start(prob)
    t = time.time()
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        y, st = s.solve(T0, TE, y0, TOL)
    t_exact = time.time() - t
    t = time.time()
    with rk.Solver(prob, method="DOPRI54", precision="mixed") as s:
        ym, stm = s.solve(T0, TE, y0, TOL)
    t_mixed = time.time() - t
    idx = sample_indices()
    rec = {
        "name": NAME, "problem": "bruss2d-mix", "grid_n": GRID_N, "alpha": ALPHA, "n": prob.n,
        "method": "DOPRI54", "tol": TOL, "t0": T0, "t_end": TE, "step_limit": 0,
        "source": "exact FP64 GPU form (rk_gb300, precision='exact'), bit-identical to the "
                  "reference on every case compared up to N=2000",
        "steps": st["steps_acc"] + st["steps_rej"], "accepted": st["steps_acc"],
        "rejected": st["steps_rej"], "step_limit_reached": False,
        "y_sha256": hashlib.sha256(y.astype("<f8").tobytes()).hexdigest(),
        "y_first": float(y[0]).hex(), "y_last": float(y[-1]).hex(),
        "y_min": float(y.min()).hex(), "y_max": float(y.max()).hex(),
        "sample": {"file": NAME + "_sample.npy", "count": int(idx.size),
                   "indices": f"rows 0 and {GRID_N - 1} in full, every {SAMPLE_STRIDE}th component"},
        "mixed": {"steps": stm["steps_acc"] + stm["steps_rej"], "accepted": stm["steps_acc"],
                  "rejected": stm["steps_rej"],
                  "rel_max_norm_full": float(np.max(np.abs(ym - y)) / np.max(np.abs(y))),
                  "rel_max_norm_sample": float(np.max(np.abs(ym[idx] - y[idx])) / np.max(np.abs(y)))},
        "seconds": {"exact": t_exact, "mixed": t_mixed},
    }
    np.save(os.path.join(a.out, NAME + "_sample.npy"), y[idx].astype("<f8"))
    with open(os.path.join(a.out, NAME + ".json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps({k: v for k, v in rec.items() if k != "sample"}))


if __name__ == "__main__":
    main()

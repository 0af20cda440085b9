"""The CPU oracle against the reference's own results (golden fixtures).

Every fixture in tests/golden was produced by the reference solver compiled
from its sources (tests/golden/make_golden.py).  The oracle must reproduce
step counts, the per-step h sequence and every stored component bit for bit.
"""
import hashlib

import numpy as np
import pytest

from conftest import all_golden, golden_y, golden_y0

# keep the CPU suite within a few minutes: component-steps per case
CPU_BUDGET = 2.5e8
CASES = [g for g in all_golden() if g["n"] * g["steps"] <= CPU_BUDGET]


def _kind(rec, oracle):
    return oracle.BRUSS2D_MIX if rec["problem"] == "bruss2d-mix" else oracle.LV_PAIRS


@pytest.mark.parametrize("rec", CASES, ids=[g["name"] for g in CASES])
def test_oracle_matches_reference(rec, oracle):
    y0 = golden_y0(rec)
    threads = 4 if rec["n"] * rec["steps"] > 5e6 else 1
    y, st = oracle.solve(_kind(rec, oracle), y0, rec["method"], rec["t0"], rec["t_end"], rec["tol"],
                         step_limit=rec["step_limit"], grid_n=rec.get("grid_n", 0),
                         alpha=rec.get("alpha", 0.0), threads=threads, trace=True)
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    if "h_trace" in rec:
        ref_h = np.array([float.fromhex(x) for x in rec["h_trace"]])
        np.testing.assert_array_equal(st["h_trace"], ref_h)
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]
    idx, vals = golden_y(rec)
    np.testing.assert_array_equal(y[idx], vals)
    assert float(y[0]).hex() == rec["y_first"] and float(y[-1]).hex() == rec["y_last"]
    assert float(y.min()).hex() == rec["y_min"] and float(y.max()).hex() == rec["y_max"]


def test_threaded_oracle_is_bit_identical(oracle):
    y0 = oracle.bruss_start(40)
    a, sa = oracle.solve(oracle.BRUSS2D_MIX, y0, "DOPRI54", 0.0, 0.2, 1e-6, grid_n=40, alpha=2e-3,
                         threads=1)
    b, sb = oracle.solve(oracle.BRUSS2D_MIX, y0, "DOPRI54", 0.0, 0.2, 1e-6, grid_n=40, alpha=2e-3,
                         threads=5)
    assert sa == sb
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("method,threads", [("DOPRI54", 1), ("DOPRI54", 3), ("DOPRI87", 2),
                                            ("RKF23", 4)])
def test_pipelined_oracle_is_bit_identical(oracle, method, threads):
    """The cache-blocked (pipelined) schedule used as the CPU baseline gives the D schedule's bits."""
    y0 = oracle.bruss_start(48)
    a, sa = oracle.solve(oracle.BRUSS2D_MIX, y0, method, 0.0, 0.2, 1e-6, grid_n=48, alpha=2e-3,
                         threads=1)
    b, sb = oracle.solve(oracle.BRUSS2D_MIX, y0, method, 0.0, 0.2, 1e-6, grid_n=48, alpha=2e-3,
                         threads=threads, rows=1)
    assert sa == sb
    np.testing.assert_array_equal(a, b)


def test_oracle_rejects_bad_arguments(oracle):
    y0 = oracle.bruss_start(8)
    with pytest.raises(RuntimeError):   # fixed step size needs a step limit
        oracle.solve(oracle.BRUSS2D_MIX, y0, "RK4", 0.0, 0.1, 0.0, step_limit=0, grid_n=8, alpha=2e-3)
    with pytest.raises(RuntimeError):   # n != 2 N^2
        oracle.solve(oracle.BRUSS2D_MIX, y0[:-2], "DOPRI54", 0.0, 0.1, 1e-6, grid_n=8, alpha=2e-3)


def test_oracle_planted_mistake_is_caught(oracle):
    """A perturbed initial value must change the pinned result (the comparison has teeth)."""
    rec = [g for g in CASES if g["name"] == "bruss_n16_a1e-2_tol1e-8"][0]
    y0 = golden_y0(rec)
    y0[37] = np.nextafter(y0[37], 2.0)
    y, _ = oracle.solve(oracle.BRUSS2D_MIX, y0, rec["method"], 0.0, rec["t_end"], rec["tol"],
                        grid_n=rec["grid_n"], alpha=rec["alpha"])
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() != rec["y_sha256"]

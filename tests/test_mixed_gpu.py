"""Mixed-precision form: FP32 stage vectors, FP64 state, update and error norm.

Bar: the result stays within the requested tolerance (relative max-norm) of the
FP64 reference/oracle, and the error is stated for each case.
"""
import json
import os
import sys

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import golden_y, golden_y0, load_golden

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", ["bruss_n250_dopri54_tol1e-6", "bruss_n100_dopri54_tol1e-6",
                                  "bruss_n250_dopri87_tol1e-6", "bruss_n2000_dopri54_tol1e-6"])
def test_mixed_within_tolerance_of_reference(name):
    rec = load_golden(name)
    y0 = golden_y0(rec)
    with rk.Solver(rk.bruss2d_mix(rec["grid_n"], rec["alpha"]), method=rec["method"],
                   precision="mixed") as s:
        y, st = s.solve(0.0, rec["t_end"], y0, rec["tol"])
    idx, ref = golden_y(rec)
    err = _rel(y[idx], ref)
    print(f"{name}: mixed steps {st['steps_acc']}+{st['steps_rej']} "
          f"(reference {rec['accepted']}+{rec['rejected']}), rel error {err:.3e}")
    assert err <= rec["tol"]
    assert abs(st["steps_acc"] + st["steps_rej"] - rec["steps"]) <= max(3, rec["steps"] // 10)


def test_mixed_full_size_short_interval_against_fp64():
    """N=4000 (n = 32e6), the mixed configuration's size, over t in [0, 0.004]:
    mixed against the exact FP64 path (itself bit-identical to the reference)."""
    N, te, tol = 4000, 0.004, 1e-6
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        ref, rst = s.solve(0.0, te, y0, tol)
    with rk.Solver(prob, method="DOPRI54", precision="mixed") as s:
        y, st = s.solve(0.0, te, y0, tol)
    err = _rel(y, ref)
    print(f"N=4000 t=[0,{te}]: mixed {st['steps_acc']}+{st['steps_rej']}, "
          f"fp64 {rst['steps_acc']}+{rst['steps_rej']}, rel error {err:.3e}")
    assert err <= tol


N4000 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "n4000",
                     "bruss_n4000_dopri54_tol1e-6")


def n4000_fixture():
    """The FP64 final state of the N=4000 solve at its stored sample indices
    (tests/golden/make_n4000_fixture.py) and the fixture's record."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(N4000)))  # tests/golden
    with open(N4000 + ".json") as f:
        rec = json.load(f)
    from make_n4000_fixture import sample_indices
    return rec, sample_indices(rec["grid_n"]), np.load(N4000 + "_sample.npy")


def test_mixed_n4000_full_interval_against_fp64_fixture():
    """The mixed configuration itself: N=4000 (n = 32e6), DOPRI5(4), tol 1e-6,
    t in [0, 0.5] (about 4e4 steps), against the final state of the exact FP64
    form (bit-identical to the reference wherever compared) at the fixture's
    sample: the first and last grid rows and every 977th component."""
    rec, idx, ref = n4000_fixture()
    prob = rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    y0 = rk.ode_start(prob)
    with rk.Solver(prob, method="DOPRI54", precision="mixed") as s:
        y, st = s.solve(rec["t0"], rec["t_end"], y0, rec["tol"])
    err = float(np.max(np.abs(y[idx] - ref)) / np.max(np.abs(ref)))
    print(f"N=4000 t=[0,0.5]: mixed {st['steps_acc']}+{st['steps_rej']}, "
          f"fp64 {rec['accepted']}+{rec['rejected']}, rel error on the sample {err:.3e}")
    assert st["t"] == rec["t_end"]
    assert err <= rec["tol"]
    assert abs(st["steps_acc"] + st["steps_rej"] - rec["steps"]) <= max(3, rec["steps"] // 10)


def test_mixed_fp64_fallback_points_within_tolerance():
    """Grid points whose values the double-float evaluation of F0 does not
    cover take the FP64 evaluation: zeros (both signs), a subnormal and
    magnitudes below 2^-80 planted in y0 (u and v components; interior, edge and
    corner points, so their stencil neighbours see them too).  Twenty fixed
    steps (tol 0: h = 0.1 / 20, as initial_stepsize gives without a tolerance)
    of the mixed form agree with the exact FP64 form to 1e-6 relative max-norm
    at the same t."""
    N, te, steps = 64, 0.1, 20
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    planted = {2 * (N * 10 + 10): 0.0, 2 * (N * 10 + 11) + 1: 0.0, 2 * (N * 30 + 40): 1e-30,
               2 * (N * 31 + 40) + 1: 5e-320, 0: 0.0, 2 * (N * N - 1) + 1: 1e-26,
               2 * (N * 63 + 20): -0.0, 2 * (N * 5 + 0) + 1: 3e-40}
    for i, v in planted.items():
        y0[i] = v
    out = {}
    for prec in ("exact", "mixed"):
        with rk.Solver(prob, method="DOPRI54", precision=prec, step_limit=steps) as s:
            out[prec] = s.solve(0.0, te, y0, 0.0)
    (ref, rst), (y, st) = out["exact"], out["mixed"]
    err = _rel(y, ref)
    print(f"planted fallback points: {steps} fixed steps to t={st['t']:.3e}, rel error {err:.3e}")
    assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"]) == (steps, 0)
    assert st["t"] == rst["t"]
    assert np.all(np.isfinite(y))
    assert err <= 1e-6


def test_mixed_rejects_problems_without_a_mixed_evaluator():
    with pytest.raises(rk.RkcuError) as ei:
        rk.Solver(rk.lv_pairs(100), precision="mixed")
    assert ei.value.status == rk.ERR_INVALID


@pytest.mark.parametrize("N,method", [(64, "DOPRI54"), (250, "DOPRI54"), (48, "RKF23"),
                                      (40, "DOPRI87"), (37, "DOPRI54"), (2, "DOPRI54"),
                                      (66, "VERNER65"), (34, "HEUN2"), (100, "RK4")])
def test_mixed_paths_give_the_same_bits(N, method):
    """The FP32 stages run all together per 32 x 32 tile in shared memory
    (schedule 3, the default where it runs: even N, at most 8 stages), or one
    stage at a time over tiles staged by TMA boxes (schedule 2) or read with
    plain loads (schedule 1); every path evaluates the same operations on the
    same values, so the bits agree (also where a path falls back to another:
    odd N, 13 stages).  Tiles at the grid's edges and corners, grids smaller
    than one tile and fixed-step tableaux are among the cases."""
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    fixed = method in ("HEUN2", "RK4")
    limit, tol, te = (40, 0.0, 0.02) if fixed else (0, 1e-6, 0.1)
    out = []
    for sched in (0, 1, 2, 3):
        with rk.Solver(prob, method=method, precision="mixed", schedule=sched, step_limit=limit) as s:
            out.append(s.solve(0.0, te, y0, tol))
    (a, sa) = out[0]
    for b, sb in out[1:]:
        assert (sa["steps_acc"], sa["steps_rej"]) == (sb["steps_acc"], sb["steps_rej"])
        np.testing.assert_array_equal(a, b)


def test_mixed_odd_grid_within_tolerance():
    """An odd N (no TMA boxes: rows would not be 16-byte aligned) stays within
    the tolerance of the FP64 path."""
    N = 37
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        ref, _ = s.solve(0.0, 0.3, y0, 1e-6)
    with rk.Solver(prob, method="DOPRI54", precision="mixed") as s:
        y, _ = s.solve(0.0, 0.3, y0, 1e-6)
    assert _rel(y, ref) <= 1e-6

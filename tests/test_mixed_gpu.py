"""Mixed-precision form: FP32 stage vectors, FP64 state, update and error norm.

Bar: the result stays within the requested tolerance (relative max-norm) of the
FP64 reference/oracle, and the error is stated for each case.
"""
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


def test_mixed_rejects_problems_without_a_mixed_evaluator():
    with pytest.raises(rk.RkcuError) as ei:
        rk.Solver(rk.lv_pairs(100), precision="mixed")
    assert ei.value.status == rk.ERR_INVALID


@pytest.mark.parametrize("N,method", [(64, "DOPRI54"), (250, "DOPRI54"), (48, "RKF23"),
                                      (40, "DOPRI87"), (37, "DOPRI54")])
def test_mixed_tma_staging_equals_plain_loads(N, method):
    """The FP32 stages read their tiles through TMA boxes staged in shared
    memory (default; even N, at most 8 stages, else plain loads) or with plain
    loads (schedule 1); both evaluate the same operations on the same values,
    so the bits agree."""
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    out = []
    for sched in (0, 1):
        with rk.Solver(prob, method=method, precision="mixed", schedule=sched) as s:
            out.append(s.solve(0.0, 0.1, y0, 1e-6))
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

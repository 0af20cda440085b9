"""GPU step loop against the reference (golden fixtures) and the CPU oracle.

Bar (from the reference's contract for this path): the FP64 GPU path takes the
same accepted and rejected step counts as the reference and agrees with it to
1e-12 relative max-norm at t_end.  The exact mode keeps the reference's
rounding order; its only possible difference is the last bit of CUDA's pow()
against glibc's pow() in the step-size factor (include/tools.h:226).
"""
import numpy as np
import pytest

import rk_gb300 as rk
from conftest import all_golden, golden_y, golden_y0, load_golden

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12           # relative max-norm bound at t_end
GPU_BUDGET = 5e9          # component-steps per case in this file
CASES = [g for g in all_golden() if g["n"] * g["steps"] <= GPU_BUDGET]


def _problem(rec):
    if rec["problem"] == "bruss2d-mix":
        return rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    return rk.lv_pairs(rec["n"] // 2)


def _rel_maxnorm(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _solve(rec, precision):
    y0 = golden_y0(rec)
    with rk.Solver(_problem(rec), method=rec["method"], precision=precision,
                   step_limit=rec["step_limit"]) as s:
        y, st = s.solve(rec["t0"], rec["t_end"], y0, rec["tol"])
        assert s.launches >= 1
    return y, st


@pytest.mark.parametrize("precision", ["exact", "fma"])
@pytest.mark.parametrize("rec", CASES, ids=[g["name"] for g in CASES])
def test_solve_matches_reference(rec, precision):
    y, st = _solve(rec, precision)
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    assert bool(st["step_limit_reached"]) == rec["step_limit_reached"]
    idx, ref = golden_y(rec)
    assert _rel_maxnorm(y[idx], ref) <= REL_TOL
    assert abs(float(y.min()) - float.fromhex(rec["y_min"])) <= REL_TOL * abs(float.fromhex(rec["y_max"]))
    assert abs(float(y.max()) - float.fromhex(rec["y_max"])) <= REL_TOL * abs(float.fromhex(rec["y_max"]))


@pytest.mark.parametrize("name", ["bruss_n16_a1e-2_tol1e-8", "bruss_n2_dopri54", "bruss_n5_dopri87",
                                  "bruss_n32_rk4_fixed", "lv_pairs_1000_dopri54"])
def test_exact_mode_is_bit_identical(name):
    """Exact mode reproduces the reference bit for bit on these cases (CUDA and glibc
    pow() agree on every step-size factor they meet)."""
    rec = load_golden(name)
    y, st = _solve(rec, "exact")
    idx, ref = golden_y(rec)
    np.testing.assert_array_equal(y[idx], ref)


@pytest.mark.parametrize("N", [2, 3, 4, 7, 64, 250])
def test_bruss_rhs_bit_exact(N, oracle):
    rng = np.random.default_rng(N)
    y = rng.uniform(0.3, 5.5, 2 * N * N)
    prob = rk.bruss2d_mix(N, 3e-3)
    f = rk.ode_eval_rng(prob, 0, prob.n - 1, 0.0, y)
    ref = oracle.eval_all(oracle.BRUSS2D_MIX, y, grid_n=N, alpha=3e-3)
    np.testing.assert_array_equal(f, ref)


def test_rhs_range_semantics(oracle):
    """ode_eval_rng(i, j) fills f[i..j] only, with global indexing (include/ode.h:34)."""
    N = 9
    y = np.random.default_rng(1).uniform(0.5, 2.0, 2 * N * N)
    prob = rk.bruss2d_mix(N, 2e-3)
    f = rk.ode_eval_rng(prob, 5, 40, 0.0, y)
    ref = oracle.eval_all(oracle.BRUSS2D_MIX, y, grid_n=N, alpha=2e-3)
    np.testing.assert_array_equal(f[5:41], ref[5:41])
    assert not f[:5].any() and not f[41:].any()


def test_lv_rhs_bit_exact(oracle):
    y = np.random.default_rng(2).uniform(0.1, 2.0, 2000)
    f = rk.ode_eval_rng(rk.lv_pairs(1000), 0, 1999, 0.0, y)
    np.testing.assert_array_equal(f, oracle.eval_all(oracle.LV_PAIRS, y))
    for n in (5, 6, 1001):
        prob, y0 = rk.lv_banded_random(n, seed=n)
        f = rk.ode_eval_rng(prob, 0, n - 1, 0.0, y0)
        ref = oracle.eval_all(oracle.LV_BANDED, y0, lv_r=prob.lv_r, lv_a=prob.lv_a)
        np.testing.assert_array_equal(f, ref)


@pytest.mark.parametrize("n", [7, 1000, 4096])
def test_banded_lv_solve_matches_oracle(n, oracle):
    """The banded chain has no reference module; the oracle's restatement of the
    reference's solver (seq/D.c) driving the chain is the check."""
    prob, y0 = rk.lv_banded_random(n, seed=100 + n)
    ref, rst = oracle.solve(oracle.LV_BANDED, y0, "DOPRI54", 0.0, 10.0, 1e-6,
                            lv_r=prob.lv_r, lv_a=prob.lv_a)
    for precision in ("exact", "fma"):
        with rk.Solver(prob, method="DOPRI54", precision=precision) as s:
            y, st = s.solve(0.0, 10.0, y0, 1e-6)
        assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])
        assert _rel_maxnorm(y, ref) <= REL_TOL


def test_device_resident_flow_equals_one_shot():
    """begin / advance(k) / query / get_y in pieces gives the one-shot result."""
    rec = load_golden("bruss_n100_dopri54_tol1e-6")
    y0 = golden_y0(rec)
    prob = _problem(rec)
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        one, st1 = s.solve(0.0, 0.5, y0, 1e-6)
        s.begin(0.0, 0.5, y0, 1e-6)
        s.advance(10)
        q = s.query()
        assert q["steps_acc"] + q["steps_rej"] == 10 and not q["done"]
        while not q["done"]:
            s.advance(7)
            q = s.query()
        np.testing.assert_array_equal(s.get_y(), one)
        assert (q["steps_acc"], q["steps_rej"]) == (st1["steps_acc"], st1["steps_rej"])


def test_solver_function_mirrors_reference_contract():
    rec = load_golden("bruss_n16_a1e-3_tol1e-4")
    y0 = golden_y0(rec)
    y = np.zeros_like(y0)
    out, st = rk.solver(0.0, 0.5, y0, y, 1e-4, problem=_problem(rec))
    assert out is y
    assert st["steps_acc"] + st["steps_rej"] == rec["steps"]


def test_wait_timeout_is_reported_and_recoverable():
    """A grid barrier waiting for CTAs that never arrive runs out of time and the
    call returns RKCU_ERR_TIMEOUT; the context stays usable for the next solve."""
    rec = load_golden("bruss_n16_a1e-2_tol1e-8")
    y0 = golden_y0(rec)
    with rk.Solver(_problem(rec), method="DOPRI54", precision="exact", wait_timeout_s=0.2) as s:
        s.inject_wait_timeout(1)
        with pytest.raises(rk.RkcuError) as ei:
            s.solve(0.0, 0.5, y0, 1e-8)
        assert ei.value.status == rk.ERR_TIMEOUT
        s.inject_wait_timeout(0)
        y, st = s.solve(0.0, 0.5, y0, 1e-8)
    idx, ref = golden_y(rec)
    assert _rel_maxnorm(y[idx], ref) <= REL_TOL
    assert st["steps_acc"] + st["steps_rej"] == rec["steps"]


def test_bad_calls_are_rejected():
    prob = rk.bruss2d_mix(8)
    with rk.Solver(prob, method="RK4") as s:
        with pytest.raises(rk.RkcuError) as ei:   # fixed step needs STEP_LIMIT > 0
            s.solve(0.0, 0.1, rk.ode_start(prob), 0.0)
        assert ei.value.status == rk.ERR_INVALID
        with pytest.raises(rk.RkcuError) as ei:
            s.advance(3)                          # nothing begun
        assert ei.value.status == rk.ERR_STATE

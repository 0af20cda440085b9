"""GPU step loop against the reference (golden fixtures) and the CPU oracle.

Bar: the FP64 GPU path takes the same accepted and rejected step counts as the
reference and agrees with it to 1e-12 relative max-norm at t_end.  The exact
mode keeps the reference's rounding order and its step-size updates (with the
C library's pow where a correctly rounded pow could differ), so it is held to
bit identity.  The FMA mode rounds differently; stiff problems near their
stability limit amplify round-off into different accept/reject decisions, so it
is held to the tolerance the solve asks for, not to step counts.
"""
import hashlib

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


@pytest.mark.parametrize("rec", CASES, ids=[g["name"] for g in CASES])
def test_exact_mode_matches_reference(rec):
    """Same step counts, the 1e-12 bar, and in fact every stored component bit for bit."""
    y, st = _solve(rec, "exact")
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    assert bool(st["step_limit_reached"]) == rec["step_limit_reached"]
    idx, ref = golden_y(rec)
    assert _rel_maxnorm(y[idx], ref) <= REL_TOL
    np.testing.assert_array_equal(y[idx], ref)
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]


@pytest.mark.parametrize("rec", CASES, ids=[g["name"] for g in CASES])
def test_fma_mode_within_tolerance(rec):
    """FMA mode: the result stays within the solve's own accuracy of the reference."""
    y, st = _solve(rec, "fma")
    idx, ref = golden_y(rec)
    tol = rec["tol"] if rec["tol"] > 0 else 1e-6
    assert _rel_maxnorm(y[idx], ref) <= 10 * tol
    steps = st["steps_acc"] + st["steps_rej"]
    assert abs(steps - rec["steps"]) <= max(2, rec["steps"] // 20)


def test_device_step_sizes_equal_host(oracle):
    """The device controller's step-size updates equal the host copy bit for bit,
    flags included, and agree with this host's C library wherever no flag is raised."""
    rng = np.random.default_rng(5)
    err = 10 ** rng.uniform(-9, -3, 20000)
    h = 10 ** rng.uniform(-7, -3, err.size)
    for ord_ in (2, 5, 8):
        dv, dflag = rk.step_sizes(h, err, 1e-6, ord_, device=True)
        hv, hflag = rk.step_sizes(h, err, 1e-6, ord_, device=False)
        np.testing.assert_array_equal(dv, hv)
        np.testing.assert_array_equal(dflag, hflag)
        libc = np.array([oracle.h_new(a, b, 1e-6, ord_) for a, b in zip(h, err)])
        assert np.all((dv == libc) | dflag)


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
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        y, st = s.solve(0.0, 10.0, y0, 1e-6)
    assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])
    np.testing.assert_array_equal(y, ref)
    with rk.Solver(prob, method="DOPRI54", precision="fma") as s:
        y, st = s.solve(0.0, 10.0, y0, 1e-6)
    assert _rel_maxnorm(y, ref) <= 1e-5


def test_device_resident_flow_equals_one_shot():
    """begin / advance(k) / query / get_y in pieces gives the one-shot result."""
    rec = load_golden("bruss_n100_dopri54_tol1e-6")
    y0 = golden_y0(rec)
    prob = _problem(rec)
    with rk.Solver(prob, method="DOPRI54", precision="exact") as s:
        one, st1 = s.solve(0.0, 0.5, y0, 1e-6)
        s.begin(0.0, 0.5, y0, 1e-6)
        q = s.run(10)
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


@pytest.mark.parametrize("cfg", [dict(schedule=1), dict(schedule=3), dict(schedule=4),
                                 dict(variant=rk.VARIANT_LOWSTORAGE), dict(precision="mixed"),
                                 dict(precision="mixed", schedule=2),
                                 dict(precision="mixed", schedule=1)],
                         ids=["grid-barrier", "flow-tiles", "row-ring", "low-storage", "mixed-fused",
                              "mixed-tma-tiles", "mixed-plain-loads"])
def test_wait_timeout_in_every_persistent_kernel(cfg):
    """Each persistent kernel's bounded waits end with RKCU_ERR_TIMEOUT when CTAs
    that never exist are awaited; the next solve on the same solver then equals
    a fresh solver's result bit for bit."""
    prob = rk.bruss2d_mix(16, 1e-2)
    y0 = rk.ode_start(prob)
    kw = dict(method="DOPRI54", **cfg)
    with rk.Solver(prob, **kw) as ref_solver:
        ref, rst = ref_solver.solve(0.0, 0.3, y0, 1e-7)
    with rk.Solver(prob, wait_timeout_s=0.2, **kw) as s:
        s.inject_wait_timeout(1)
        with pytest.raises(rk.RkcuError) as ei:
            s.solve(0.0, 0.3, y0, 1e-7)
        assert ei.value.status == rk.ERR_TIMEOUT
        s.inject_wait_timeout(0)
        y, st = s.solve(0.0, 0.3, y0, 1e-7)
    assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])
    np.testing.assert_array_equal(y, ref)


def test_bad_calls_are_rejected():
    prob = rk.bruss2d_mix(8)
    with rk.Solver(prob, method="RK4") as s:
        with pytest.raises(rk.RkcuError) as ei:   # fixed step needs STEP_LIMIT > 0
            s.solve(0.0, 0.1, rk.ode_start(prob), 0.0)
        assert ei.value.status == rk.ERR_INVALID
        with pytest.raises(rk.RkcuError) as ei:
            s.advance(3)                          # nothing begun
        assert ei.value.status == rk.ERR_STATE


@pytest.mark.parametrize("name", ["bruss_n250_dopri54_tol1e-6", "bruss_n64_dopri87_tol1e-7",
                                  "lv_pairs_1000_dopri54"])
def test_products_on_integer_pipe_equal_fp64_pipe(name):
    """The default exact mode computes products on the integer pipe; with every
    product on the FP64 pipe the results are the same bit for bit."""
    rec = load_golden(name)
    a, sa = _solve(rec, "exact")
    for other in ("exact-hwmul",):
        b, sb = _solve(rec, other)
        np.testing.assert_array_equal(a, b)
        assert (sa["steps_acc"], sa["steps_rej"]) == (sb["steps_acc"], sb["steps_rej"])
    assert hashlib.sha256(a.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]

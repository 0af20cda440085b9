"""General right-hand sides (RKCU_PROBLEM_RHS): the step loop of the
reference's A variant (src/impl/seq/A.c:57-85) around a device function the
caller supplies.

With the built-in modules as that function (rkcu_rhs_builtin) the exact mode
must reproduce the reference's golden results bit for bit; with a Python
function on torch tensors (a non-autonomous system and a dense coupling, which
no stencil kernel can serve) it must reach the solve's tolerance against the
analytic solution.
"""
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import golden_y0, load_golden

pytestmark = pytest.mark.gpu

GOLDEN = ["bruss_n2_dopri54", "bruss_n8_dopri54", "bruss_n16_a1e-2_tol1e-8", "bruss_n32_rkf23",
          "bruss_n32_rk4_fixed", "bruss_n32_steplimit20", "bruss_n64_dopri87_tol1e-7",
          "bruss_n250_dopri54_tol1e-6", "lv_pairs_1000_dopri54"]


def _builtin(rec):
    if rec["problem"] == "bruss2d-mix":
        return rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    return rk.lv_pairs(rec["n"] // 2)


@pytest.mark.parametrize("name", GOLDEN)
def test_builtin_rhs_through_general_loop_matches_reference(name):
    rec = load_golden(name)
    with rk.Solver(rk.rhs_problem(rec["n"]), method=rec["method"], precision="exact",
                   step_limit=rec["step_limit"]) as s:
        s.set_rhs("builtin", _builtin(rec))
        y, st = s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]


def _torch_rhs(body):
    import torch

    def fn(t, w, f, n, stream):
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            W = torch.as_tensor(rk.DeviceArray(w, n), device="cuda")
            F = torch.as_tensor(rk.DeviceArray(f, n), device="cuda")
            body(t, W, F)
        return 0
    return fn


def test_python_rhs_nonautonomous():
    """y' = -y + sin(t): the function receives t + h c_l for every stage."""
    import torch
    n, te, tol = 1001, 2.0, 1e-8
    y0 = np.linspace(0.0, 1.0, n)
    with rk.Solver(rk.rhs_problem(n), method="DOPRI54") as s:
        s.set_rhs(_torch_rhs(lambda t, W, F: torch.sub(torch.full_like(W, np.sin(t)), W, out=F)))
        y, st = s.solve(0.0, te, y0, tol)
    exact = (y0 + 0.5) * np.exp(-te) + 0.5 * (np.sin(te) - np.cos(te))
    assert st["done"] and np.max(np.abs(y - exact)) < 20 * tol


def test_python_rhs_dense_coupling():
    """y' = M y with a dense M (every component depends on all others), against expm."""
    import torch
    scipy_linalg = pytest.importorskip("scipy.linalg")
    n, te, tol = 256, 1.0, 1e-9
    rng = np.random.default_rng(3)
    M = -np.eye(n) + rng.standard_normal((n, n)) / (2 * np.sqrt(n))
    Mt = torch.as_tensor(M, device="cuda")
    y0 = rng.uniform(0.5, 1.5, n)
    with rk.Solver(rk.rhs_problem(n), method="DOPRI87") as s:
        s.set_rhs(_torch_rhs(lambda t, W, F: torch.mv(Mt, W, out=F)))
        y, st = s.solve(0.0, te, y0, tol)
    exact = scipy_linalg.expm(M * te) @ y0
    assert np.max(np.abs(y - exact)) / np.max(np.abs(exact)) < 50 * tol


def test_failing_rhs_stops_the_solve():
    with rk.Solver(rk.rhs_problem(10), method="DOPRI54") as s:
        s.set_rhs(lambda t, w, f, n, stream: 7)
        with pytest.raises(rk.RkcuError) as ei:
            s.solve(0.0, 1.0, np.ones(10), 1e-6)
        assert ei.value.status == rk.ERR_RHS


def test_rhs_problem_combinations_refused():
    p = rk.rhs_problem(64)
    with pytest.raises(rk.RkcuError):
        rk.Solver(p, precision="mixed")
    with pytest.raises(rk.RkcuError):
        rk.Solver(p, variant=rk.VARIANT_LOWSTORAGE)
    with rk.Solver(p) as s:
        with pytest.raises(rk.RkcuError) as ei:   # no function set yet
            s.solve(0.0, 1.0, np.ones(64), 1e-6)
        assert ei.value.status == rk.ERR_STATE
        s.set_rhs("builtin", rk.lv_pairs(32))
        with pytest.raises(rk.RkcuError):
            s.set_trace(10)
    with rk.Solver(rk.bruss2d_mix(8)) as s:
        with pytest.raises(rk.RkcuError):           # only for RKCU_PROBLEM_RHS
            s.set_rhs("builtin", rk.bruss2d_mix(8))

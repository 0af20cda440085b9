"""The allocation-free entry point rkcu_solve_noalloc, called through the C ABI.

It exists for callers that must not allocate device memory (an application
that owns all device memory through its own pool or budget, or a loop that
cannot take cudaFree's device-wide synchronisation): they pass their own
device buffers for y0 and y, and the solve keeps all of its scratch in one
static device array.  Its results must equal those of the allocating entry
point rkcu_solve, call after call, although every call reuses the array the
previous call left behind; in the exact mode they must also equal the
reference's own results (golden fixtures) bit for bit.

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import golden_y, golden_y0, load_golden

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12   # the bar the FP64 parity tests use

PRECISION = {"exact": rk.FP64_EXACT, "fma": rk.FP64_FMA}


def _reference(prob, method, te, tol, precision="exact", step_limit=0, y0=None):
    y0 = rk.ode_start(prob) if y0 is None else y0
    with rk.Solver(prob, method=method, precision=precision, step_limit=step_limit) as s:
        y, st = s.solve(0.0, te, y0, tol)
    return y0, y, st


def _noalloc(lib, prob, method, y0_dev, y_dev, te, tol, precision="exact", step_limit=0):
    st = rk.Stats()
    ps = prob.cstruct()
    rc = lib.rkcu_solve_noalloc(ctypes.byref(ps), method.encode(), PRECISION[precision], step_limit,
                                0.0, te, ctypes.c_void_p(y0_dev.data_ptr()),
                                ctypes.c_void_p(y_dev.data_ptr()), tol, None, ctypes.byref(st))
    return rc, st


def _run(lib, prob, method, y0, te, tol, precision="exact", step_limit=0):
    import torch
    y0_dev = torch.from_numpy(y0).cuda()
    y_dev = torch.full_like(y0_dev, float("nan"))
    rc, st = _noalloc(lib, prob, method, y0_dev, y_dev, te, tol, precision, step_limit)
    assert rc == rk.OK, (rc, lib.rkcu_last_cuda_error())
    torch.cuda.synchronize()
    # the input buffer is read, not written
    np.testing.assert_array_equal(y0_dev.cpu().numpy(), y0)
    return y_dev.cpu().numpy(), st


def test_noalloc_equals_allocating_entry_point_on_consecutive_calls():
    lib = rk.load()
    cases = [(rk.bruss2d_mix(64, 2e-3), "DOPRI54", 0.2, 1e-6, "exact", 0),   # n = 8192
             (rk.bruss2d_mix(64, 2e-3), "DOPRI54", 0.2, 1e-6, "exact", 0),   # the same again: stale scratch
             (rk.bruss2d_mix(23, 5e-3), "DOPRI87", 0.1, 1e-7, "exact", 0),   # smaller after larger
             (rk.bruss2d_mix(40, 2e-3), "DOPRI54", 0.2, 1e-6, "fma", 0),     # the FMA mode
             (rk.bruss2d_mix(40, 2e-3), "DOPRI54", 0.2, 1e-6, "fma", 0),
             (rk.bruss2d_mix(48, 2e-3), "DOPRI54", 0.5, 1e-8, "exact", 7),   # stopped by the step limit
             (rk.lv_pairs(32768), "DOPRI54", 2.0, 1e-6, "exact", 0)]         # n = 65536, the limit
    for prob, method, te, tol, precision, limit in cases:
        y0, ref, rst = _reference(prob, method, te, tol, precision, limit)
        y, st = _run(lib, prob, method, y0, te, tol, precision, limit)
        assert (st.steps_acc, st.steps_rej) == (rst["steps_acc"], rst["steps_rej"])
        assert bool(st.step_limit_reached) == bool(rst["step_limit_reached"]) == (limit > 0)
        rel = float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))
        assert rel <= REL_TOL, rel
        # same arithmetic as the allocating entry point: the same bits
        np.testing.assert_array_equal(y, ref)


@pytest.mark.parametrize("name", ["bruss_n100_dopri54_tol1e-6", "bruss_n16_a1e-2_tol1e-8",
                                  "bruss_n32_steplimit20", "lv_pairs_1000_dopri54"])
def test_noalloc_exact_mode_equals_reference_fixture(name):
    """Two calls in a row, each bit-identical to the reference's own run."""
    lib = rk.load()
    rec = load_golden(name)
    prob = (rk.bruss2d_mix(rec["grid_n"], rec["alpha"]) if rec["problem"] == "bruss2d-mix"
            else rk.lv_pairs(rec["n"] // 2))
    y0 = golden_y0(rec)
    idx, ref = golden_y(rec)
    for _ in range(2):
        y, st = _run(lib, prob, rec["method"], y0, rec["t_end"], rec["tol"], "exact", rec["step_limit"])
        assert (st.steps_acc, st.steps_rej) == (rec["accepted"], rec["rejected"])
        assert bool(st.step_limit_reached) == rec["step_limit_reached"]
        np.testing.assert_array_equal(y[idx], ref)
        assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]


def test_noalloc_rejects_systems_beyond_its_limit():
    import torch
    lib = rk.load()
    prob = rk.bruss2d_mix(182, 2e-3)          # n = 66248 > 65536
    buf = torch.zeros(prob.n, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(lib, prob, "DOPRI54", buf, buf, 0.1, 1e-6)
    assert rc == rk.ERR_TOO_LARGE
    assert b"65536" in lib.rkcu_strerror(rc)

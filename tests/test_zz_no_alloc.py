"""The allocation-free entry point rkcu_solve_noalloc, called through the C ABI.

It exists for callers that must not allocate device memory (an application
that owns all device memory through its own pool or budget, or a loop that
cannot take cudaFree's device-wide synchronisation): they pass their own
device buffers for y0 and y, and the solve keeps all of its scratch in one
static device array.  Its results must equal those of the allocating entry
point rkcu_solve, call after call, although every call reuses the array the
previous call left behind.

This file is collected last, so a run that stops at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import rk_gb300 as rk

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12   # the bar the FP64 parity tests use


def _reference(prob, method, te, tol):
    y0 = rk.ode_start(prob)
    with rk.Solver(prob, method=method, precision="exact") as s:
        y, st = s.solve(0.0, te, y0, tol)
    return y0, y, st


def _noalloc(lib, prob, method, y0_dev, y_dev, te, tol):
    st = rk.Stats()
    ps = prob.cstruct()
    rc = lib.rkcu_solve_noalloc(ctypes.byref(ps), method.encode(), rk.FP64_EXACT, 0, 0.0, te,
                                ctypes.c_void_p(y0_dev.data_ptr()), ctypes.c_void_p(y_dev.data_ptr()),
                                tol, None, ctypes.byref(st))
    return rc, st


def test_noalloc_equals_allocating_entry_point_on_consecutive_calls():
    import torch
    lib = rk.load()
    cases = [(rk.bruss2d_mix(64, 2e-3), "DOPRI54", 0.2, 1e-6),   # n = 8192
             (rk.bruss2d_mix(64, 2e-3), "DOPRI54", 0.2, 1e-6),   # the same again: stale scratch
             (rk.bruss2d_mix(23, 5e-3), "DOPRI87", 0.1, 1e-7),   # smaller system after a larger one
             (rk.lv_pairs(32768), "DOPRI54", 2.0, 1e-6)]         # n = 65536, the limit
    for prob, method, te, tol in cases:
        y0, ref, rst = _reference(prob, method, te, tol)
        y0_dev = torch.from_numpy(y0).cuda()
        y_dev = torch.full_like(y0_dev, float("nan"))
        rc, st = _noalloc(lib, prob, method, y0_dev, y_dev, te, tol)
        assert rc == rk.OK, rc
        torch.cuda.synchronize()
        y = y_dev.cpu().numpy()
        assert (st.steps_acc, st.steps_rej) == (rst["steps_acc"], rst["steps_rej"])
        rel = float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))
        assert rel <= REL_TOL, rel
        # the input buffer is read, not written
        np.testing.assert_array_equal(y0_dev.cpu().numpy(), y0)


def test_noalloc_rejects_systems_beyond_its_limit():
    import torch
    lib = rk.load()
    prob = rk.bruss2d_mix(182, 2e-3)          # n = 66248 > 65536
    buf = torch.zeros(prob.n, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(lib, prob, "DOPRI54", buf, buf, 0.1, 1e-6)
    assert rc == rk.ERR_TOO_LARGE
    assert b"65536" in lib.rkcu_strerror(rc)

"""The C ABI library: loads without a GPU, exports every symbol include/rkcu.h
declares, and its host-side logic (tableaux, argument checks) is right."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "rkcu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rkcu_[a-z0-9_]+)\s*\(", text)))


def test_header_and_python_exports_agree():
    import rk_gb300
    assert sorted(rk_gb300.EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol(rkcu_lib):
    missing = [s for s in declared_symbols() if not hasattr(rkcu_lib, s)]
    assert not missing, missing


@pytest.mark.parametrize("name", ["HEUN2", "RK4", "SSPRK3", "RKF23", "DOPRI54", "VERNER65", "DOPRI87"])
def test_builtin_tableaux_equal_oracle(name, rkcu_lib, oracle):
    import rk_gb300
    got = rk_gb300.builtin_method(name)
    ref = oracle.tableau(name)
    assert (got["s"], got["ord"], got["embedded"]) == (ref["s"], ref["ord"], ref["embedded"])
    for k in ("A", "b", "b_hat", "c"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


def test_unknown_method_is_rejected(rkcu_lib):
    import rk_gb300
    with pytest.raises(rk_gb300.RkcuError) as ei:
        rk_gb300.builtin_method("DOPRI99")
    assert ei.value.status == rk_gb300.ERR_INVALID


def test_strerror_and_acc_dist(rkcu_lib):
    import rk_gb300
    assert rkcu_lib.rkcu_strerror(rk_gb300.ERR_TIMEOUT) == b"device wait timed out"
    assert rk_gb300.ode_acc_dist(rk_gb300.bruss2d_mix(250)) == 500   # bruss2d-mix.c:718-721
    assert rk_gb300.ode_acc_dist(rk_gb300.lv_pairs(10)) == 1         # lv.c:127-130


def test_ode_start_matches_oracle(rkcu_lib, oracle):
    import rk_gb300
    for N in (2, 3, 17, 250):
        np.testing.assert_array_equal(rk_gb300.ode_start(rk_gb300.bruss2d_mix(N)), oracle.bruss_start(N))
    np.testing.assert_array_equal(rk_gb300.ode_start(rk_gb300.lv_pairs(7)), oracle.lv_pairs_start(14))


def test_create_validates_before_touching_a_device(rkcu_lib):
    import rk_gb300
    h = ctypes.c_void_p()
    bad = rk_gb300.Problem(rk_gb300.PROBLEM_BRUSS2D_MIX, 10, 3, 2e-3, None, None)  # n != 2N^2
    assert rkcu_lib.rkcu_create(ctypes.byref(h), ctypes.byref(bad), None) == rk_gb300.ERR_INVALID
    bad = rk_gb300.Problem(rk_gb300.PROBLEM_LV_BANDED, 10, 0, 0.0, None, None)      # no parameters
    assert rkcu_lib.rkcu_create(ctypes.byref(h), ctypes.byref(bad), None) == rk_gb300.ERR_INVALID
    assert rkcu_lib.rkcu_create(None, None, None) == rk_gb300.ERR_INVALID


def test_no_cpu_fallback_without_gpu(rkcu_lib):
    """Without a GPU the library refuses to run: it never falls back to the CPU."""
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present")
    import rk_gb300
    with pytest.raises(rk_gb300.RkcuError) as ei:
        rk_gb300.Solver(rk_gb300.bruss2d_mix(8))
    assert ei.value.status in (rk_gb300.ERR_NO_DEVICE, rk_gb300.ERR_CUDA)


def test_step_size_update_matches_c_library(rkcu_lib, oracle):
    """Host copy of the device step-size update (correctly rounded pow) equals the
    reference's h_new (include/tools.h:221-233, C library pow) wherever it does not
    ask the host to finish the update, and every disagreement is flagged."""
    import rk_gb300
    rng = np.random.default_rng(11)
    flagged = differ = unflagged_differ = 0
    for ord_ in (2, 5, 6, 8):
        err = 10 ** rng.uniform(-9, -3, 20000)
        vals, flags = rk_gb300.step_sizes(1e-5, err, 1e-6, ord_)
        for v, f, e in zip(vals, flags, err):
            ref = oracle.h_new(1e-5, e, 1e-6, ord_)
            flagged += int(f)
            if v != ref:
                differ += 1
                unflagged_differ += int(not f)
    assert unflagged_differ == 0
    assert flagged < 0.08 * 80000      # the host finishes a few percent of updates


def test_correctly_rounded_pow_against_decimal(rkcu_lib):
    """Where the C library and the device controller disagree, the controller's
    power is the correctly rounded one (60-digit decimal arithmetic decides)."""
    from decimal import Decimal, getcontext
    import rk_gb300
    getcontext().prec = 60
    rng = np.random.default_rng(3)
    err = 10 ** rng.uniform(-9, -3, 3000)
    vals, _ = rk_gb300.step_sizes(1.0, err, 1e-6, 5)
    for v, e in zip(vals, err):
        q = 1e-6 / e
        true_pow = (Decimal(q).ln() * Decimal(1.0 / 6.0)).exp()
        if Decimal("0.56") < true_pow < Decimal("2.2"):
            # with h = 1 and no clamp, v = RN(0.9 * RN(pow)): RN(pow) must be the
            # double nearest to the true power
            cand = [np.nextafter(float(true_pow), -np.inf), float(true_pow),
                    np.nextafter(float(true_pow), np.inf)]
            best = min(cand, key=lambda c: abs(Decimal(c) - true_pow))
            assert v == 0.9 * best


def test_dump_format_matches_c_printf():
    """rk_gb300.dump_text writes the reference's DUMP lines: "%.20e" as C's printf formats it."""
    import ctypes
    import ctypes.util
    import rk_gb300 as rk
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    rng = np.random.default_rng(11)
    vals = np.concatenate([rng.standard_normal(300) * 10.0 ** rng.integers(-30, 30, 300),
                           [0.0, -0.0, 1.0, 0.5, 1e-310, 1.7e308]])
    buf = ctypes.create_string_buffer(64)
    for v in vals:
        libc.snprintf(buf, 64, b"%.20e", ctypes.c_double(float(v)))
        assert ("%.20e" % v).encode() == buf.value
    tr = {"t": np.array([0.0, 0.25]), "h": np.array([0.25, 0.125]),
          "y": np.array([[1.0, 2.0], [3.0, 4.0]])}
    lines = rk.dump_text(tr).splitlines()
    assert len(lines) == 2 and lines[1].split("\t")[1] == "%.20e" % 0.125

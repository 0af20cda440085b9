"""Per-step trace of the GPU step loop against the reference's -DDUMP output.

The reference, compiled with -DDUMP, writes one line per attempted step from
step_control (include/tools.h:239-256): t, h and every component of the step's
candidate state as %.20e.  The golden fixtures hold the t and h of every line
and, for small systems, the sha256 of the whole DUMP file.  The GPU path's
trace (rkcu_set_trace / rkcu_get_trace), written in the same format, must
reproduce those bytes.
"""
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import all_golden, golden_y0

pytestmark = pytest.mark.gpu

TRACED = [g for g in all_golden() if "t_trace" in g]
DUMPED = [g for g in TRACED if "dump_sha256" in g]


def _problem(rec):
    if rec["problem"] == "bruss2d-mix":
        return rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    return rk.lv_pairs(rec["n"] // 2)


def _traced_solve(rec, with_y):
    with rk.Solver(_problem(rec), method=rec["method"], precision="exact",
                   step_limit=rec["step_limit"]) as s:
        s.set_trace(rec["steps"] + 4, with_y=with_y)
        y, st = s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])
        return y, st, s.trace()


@pytest.mark.parametrize("rec", TRACED, ids=[g["name"] for g in TRACED])
def test_trace_t_and_h_equal_reference_dump(rec):
    y, st, tr = _traced_solve(rec, with_y=False)
    assert len(tr["h"]) == rec["steps"]
    assert [float(v).hex() for v in tr["h"]] == rec["h_trace"]
    assert [float(v).hex() for v in tr["t"]] == rec["t_trace"]
    # an accepted step's error max is within tol, a rejected one's above it
    if rec["tol"] > 0:
        acc = np.diff(np.append(tr["t"], st["t"])) != 0
        assert np.all(tr["err"][acc] <= rec["tol"]) and np.all(tr["err"][~acc] > rec["tol"])


@pytest.mark.parametrize("rec", DUMPED, ids=[g["name"] for g in DUMPED])
def test_dump_file_bytes_equal_reference(rec):
    y, st, tr = _traced_solve(rec, with_y=True)
    text = rk.dump_text(tr).encode()
    assert len(text) == rec["dump_bytes"]
    assert hashlib.sha256(text).hexdigest() == rec["dump_sha256"]
    # the last candidate is the final state when the last step was accepted
    if st["t"] != tr["t"][-1]:
        np.testing.assert_array_equal(tr["y"][-1], y)


def test_trace_capacity_truncates_and_resets():
    rec = DUMPED[0]
    p = _problem(rec)
    y0 = golden_y0(rec)
    with rk.Solver(p, method=rec["method"], precision="exact") as s:
        s.set_trace(5, with_y=True)
        s.solve(rec["t0"], rec["t_end"], y0, rec["tol"])
        tr = s.trace()
        assert len(tr["t"]) == 5 and tr["y"].shape == (5, p.n)
        assert [float(v).hex() for v in tr["h"]] == rec["h_trace"][:5]
        s.set_trace(0)
        s.solve(rec["t0"], rec["t_end"], y0, rec["tol"])
        assert len(s.trace()["t"]) == 0


def test_trace_refused_outside_plain_fp64_form():
    p = rk.bruss2d_mix(16, 2e-3)
    with rk.Solver(p, precision="mixed") as s:
        with pytest.raises(rk.RkcuError):
            s.set_trace(10)
    with rk.Solver(p, variant=rk.VARIANT_LOWSTORAGE) as s:
        with pytest.raises(rk.RkcuError):
            s.set_trace(10)

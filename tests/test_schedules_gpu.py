"""Stage-synchronisation schedules of the plain kernel give identical bits.

The plain kernel can close a stage with a grid barrier (schedule 1), with
neighbour progress flags (2, also the automatic choice 0 that the other tests
use), or run a dataflow over (stage, tile) tickets in wavefront order (3), or
stage each stage input's grid rows in a shared-memory ring by bulk copies (4,
BRUSS2D-MIX; LV falls back to 2).  Every schedule applies the same operations in the same
order to every component, so the exact mode must reproduce the reference's
golden results bit for bit under each, for any tile size and skew.
"""
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import golden_y0, load_golden

pytestmark = pytest.mark.gpu

GOLDEN = ["bruss_n2_dopri54", "bruss_n3_dopri54", "bruss_n8_dopri54", "bruss_n16_a1e-2_tol1e-8",
          "bruss_n32_rkf23", "bruss_n32_verner65", "bruss_n32_steplimit20", "bruss_n64_dopri87_tol1e-7",
          "bruss_n100_dopri54_tol1e-6", "bruss_n250_dopri54_tol1e-6", "lv_pairs_1000_dopri54"]


def _problem(rec):
    if rec["problem"] == "bruss2d-mix":
        return rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    return rk.lv_pairs(rec["n"] // 2)


def _solve(rec, **kw):
    with rk.Solver(_problem(rec), method=rec["method"], precision=kw.pop("precision", "exact"),
                   step_limit=rec["step_limit"], **kw) as s:
        return s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])


@pytest.mark.parametrize("name", GOLDEN)
@pytest.mark.parametrize("sched", [
    dict(schedule=1),
    dict(schedule=3),
    dict(schedule=3, flow_skew=1),
    dict(schedule=3, flow_skew=5, block_rows=2),
    dict(schedule=4),
], ids=["grid-barrier", "flow-auto", "flow-k1", "flow-k5-r2", "row-ring"])
def test_schedule_matches_reference(name, sched):
    rec = load_golden(name)
    y, st = _solve(rec, **sched)
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]


@pytest.mark.parametrize("sched", [dict(schedule=1), dict(schedule=2), dict(schedule=3),
                                   dict(schedule=3, flow_skew=2)])
def test_schedules_agree_on_banded_lv(sched):
    p, y0 = rk.lv_banded_random(50000, seed=3)
    with rk.Solver(p, method="DOPRI54", precision="exact") as s:
        ref, sref = s.solve(0.0, 2.0, y0, 1e-6)
    with rk.Solver(p, method="DOPRI54", precision="exact", **sched) as s:
        y, st = s.solve(0.0, 2.0, y0, 1e-6)
    assert (st["steps_acc"], st["steps_rej"]) == (sref["steps_acc"], sref["steps_rej"])
    np.testing.assert_array_equal(y, ref)


def test_flow_schedule_fma_and_trace():
    """The flow schedule also serves the FMA mode and the per-step trace."""
    rec = load_golden("bruss_n32_rkf23")
    a, sa = _solve(rec, precision="fma", schedule=1)
    b, sb = _solve(rec, precision="fma", schedule=3)
    np.testing.assert_array_equal(a, b)
    with rk.Solver(_problem(rec), method=rec["method"], schedule=3) as s:
        s.set_trace(rec["steps"], with_y=False)
        s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])
        assert [float(v).hex() for v in s.trace()["h"]] == rec["h_trace"]


def test_row_ring_fma_trace_and_n2000():
    """The row ring also serves the FMA mode and the per-step trace, and at the
    FP64 configuration's size its steps equal the default schedule's bit for bit."""
    rec = load_golden("bruss_n32_rkf23")
    a, _ = _solve(rec, precision="fma")
    b, _ = _solve(rec, precision="fma", schedule=4)
    np.testing.assert_array_equal(a, b)
    with rk.Solver(_problem(rec), method=rec["method"], schedule=4) as s:
        s.set_trace(rec["steps"], with_y=False)
        s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])
        assert [float(v).hex() for v in s.trace()["h"]] == rec["h_trace"]
    prob = rk.bruss2d_mix(2000, 2e-3)
    y0 = rk.ode_start(prob)
    out = []
    for sched in (0, 4):
        with rk.Solver(prob, method="DOPRI54", precision="exact", schedule=sched, step_limit=40) as s:
            out.append(s.solve(0.0, 0.5, y0, 1e-6))
    assert (out[0][1]["steps_acc"], out[0][1]["steps_rej"]) == (out[1][1]["steps_acc"], out[1][1]["steps_rej"])
    np.testing.assert_array_equal(out[0][0], out[1][0])

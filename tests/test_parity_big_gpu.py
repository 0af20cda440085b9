"""The N=2000 FP64 configuration against the reference's own full runs.

The fixtures hold the reference's step counts and a sample of its final state
(pthreads PipeD4ls, bit-identical to seq D) for DOPRI5(4) and DOPRI8(7); the
exact mode must reproduce both bit for bit (sha256 of all 8,000,000 components).
"""
import hashlib
import os

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import GOLDEN, golden_y, golden_y0, load_golden

pytestmark = pytest.mark.gpu

NAMES = [n for n in ("bruss_n2000_dopri54_tol1e-6", "bruss_n2000_dopri87_tol1e-6")
         if os.path.exists(os.path.join(GOLDEN, n + ".json"))]


@pytest.mark.parametrize("name", NAMES)
def test_n2000_exact_matches_reference(name):
    rec = load_golden(name)
    y0 = golden_y0(rec)
    with rk.Solver(rk.bruss2d_mix(rec["grid_n"], rec["alpha"]), method=rec["method"],
                   precision="exact") as s:
        y, st = s.solve(0.0, rec["t_end"], y0, rec["tol"])
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    idx, ref = golden_y(rec)
    rel = float(np.max(np.abs(y[idx] - ref)) / np.max(np.abs(ref)))
    assert rel <= 1e-12
    np.testing.assert_array_equal(y[idx], ref)
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]

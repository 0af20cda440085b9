"""Low-storage (pipelined wavefront) variant: bit-identical to the reference and
to the plain form for any block size, with 2n + O(s^2 B) device storage."""
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import all_golden, golden_y, golden_y0, load_golden

pytestmark = pytest.mark.gpu

CASES = [g for g in all_golden() if g["problem"] == "bruss2d-mix" and g["n"] * g["steps"] <= 5e9]


def _solve(rec, rows, precision="exact"):
    with rk.Solver(rk.bruss2d_mix(rec["grid_n"], rec["alpha"]), method=rec["method"],
                   precision=precision, step_limit=rec["step_limit"],
                   variant=rk.VARIANT_LOWSTORAGE, block_rows=rows) as s:
        y, st = s.solve(rec["t0"], rec["t_end"], golden_y0(rec), rec["tol"])
        return y, st, s.device_bytes


@pytest.mark.parametrize("rows", [0, 1, 3])
@pytest.mark.parametrize("rec", CASES, ids=[g["name"] for g in CASES])
def test_lowstorage_bit_identical_to_reference(rec, rows):
    y, st, _ = _solve(rec, rows)
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    idx, ref = golden_y(rec)
    np.testing.assert_array_equal(y[idx], ref)
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]


def test_lowstorage_n2000_matches_reference_with_less_memory():
    rec = load_golden("bruss_n2000_dopri54_tol1e-6")
    y, st, ls_bytes = _solve(rec, 0)
    assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"])
    assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"]
    n = rec["n"]
    # 2n state doubles + the ring window: 2n + (s^2 + 5s - 4) R 2N doubles with
    # blocks of R = 64 rows (128 MB + 164 MB), against the plain form's (s+3) n
    N, s, R = rec["grid_n"], 7, 64
    assert ls_bytes == (2 * n + (s * s + 5 * s - 4) * R * 2 * N) * 8
    assert ls_bytes < 0.5 * (s + 3) * n * 8
    print(f"low-storage device bytes {ls_bytes / 1e6:.0f} MB vs plain {(7 + 3) * n * 8 / 1e6:.0f} MB")


@pytest.mark.parametrize("method", ["DOPRI54", "DOPRI87"])
def test_lowstorage_fma_equals_plain_fma(method):
    """The FMA mode applies the same operations per component in both forms."""
    prob = rk.bruss2d_mix(64, 5e-3)
    y0 = rk.ode_start(prob)
    out = []
    for variant in (rk.VARIANT_D, rk.VARIANT_LOWSTORAGE):
        with rk.Solver(prob, method=method, precision="fma", variant=variant) as s:
            out.append(s.solve(0.0, 0.2, y0, 1e-7))
    (a, sa), (b, sb) = out
    assert (sa["steps_acc"], sa["steps_rej"]) == (sb["steps_acc"], sb["steps_rej"])
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("N,rows,method", [(2000, 0, "DOPRI54"), (300, 64, "DOPRI54"), (7, 2, "DOPRI54"),
                                           (2, 1, "DOPRI54"), (150, 32, "DOPRI87")])
def test_lowstorage_neighbour_flags_equal_grid_barrier(N, rows, method):
    """The neighbour-flag synchronisation between wavefront steps (the default) and a
    grid barrier per step give the same bits: blocks that do not divide the grid
    (N=2000 with R=64 leaves a 16-row last block), CTAs without work (tiny grids), and
    the 13-stage tableau."""
    prob = rk.bruss2d_mix(N, 2e-3)
    y0 = rk.ode_start(prob)
    te = 0.002 if N >= 1000 else 0.05
    out = []
    for schedule in (0, 1):
        with rk.Solver(prob, method=method, variant=rk.VARIANT_LOWSTORAGE, block_rows=rows,
                       schedule=schedule) as s:
            out.append(s.solve(0.0, te, y0, 1e-6))
    (a, sa), (b, sb) = out
    assert (sa["steps_acc"], sa["steps_rej"]) == (sb["steps_acc"], sb["steps_rej"])
    np.testing.assert_array_equal(a, b)
    with rk.Solver(prob, method=method, schedule=0) as s:
        c, sc = s.solve(0.0, te, y0, 1e-6)
    np.testing.assert_array_equal(a, c)


def test_lowstorage_rejects_other_problems():
    with pytest.raises(rk.RkcuError) as ei:
        rk.Solver(rk.lv_pairs(10), variant=rk.VARIANT_LOWSTORAGE)
    assert ei.value.status == rk.ERR_INVALID

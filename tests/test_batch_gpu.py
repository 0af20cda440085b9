"""Batched step loop: many uneven instances in one persistent launch.

Checks: every instance's result is the same alone and in the mix (bit for
bit) and, in the exact mode, equal to the reference's own result (golden
fixtures) or to the oracle bit for bit with the same step counts -- step-size
factors near a rounding boundary are answered by the host with the C
library's pow, as in the plain form; the autotuner and the graph replay change
nothing, and admission by HBM footprint refuses what does not fit and admits
it after space is freed.
"""
import hashlib

import numpy as np
import pytest

import rk_gb300 as rk
from conftest import golden_y, golden_y0, load_golden
from rk_gb300 import workloads

pytestmark = pytest.mark.gpu

GB = 1 << 30


def _mix(seed=3):
    """A small, uneven mix: BRUSS2D-MIX of several sizes/tolerances, LV pairs, banded LV."""
    rng = np.random.default_rng(seed)
    items = []
    for k in range(18):
        N = int(rng.integers(2, 48))
        a = float(rng.uniform(1e-3, 1e-2))
        tol = float(np.exp(rng.uniform(np.log(1e-8), np.log(1e-4))))
        p = rk.bruss2d_mix(N, a)
        items.append((p, rk.ode_start(p), 0.0, 0.5, tol))
    for cnt in (3, 50, 700):
        p = rk.lv_pairs(cnt)
        items.append((p, rk.ode_start(p), 0.0, 10.0, 1e-6))
    for n in (5, 333, 2000):
        p, y0 = rk.lv_banded_random(n, seed=n)
        items.append((p, y0, 0.0, 10.0, 1e-6))
    return items


def _run_batch(items, tune=False, graph=True, sweeps=64, precision="exact"):
    out = {}
    with rk.Batch(1 * GB, 64, precision=precision) as b:
        if not graph:
            b.set_tuning(256, 512, 0, use_graph=False)
        for k, (p, y0, t0, te, tol) in enumerate(items):
            assert b.add(p, y0, t0, te, tol, host_id=k) is not None
        if tune:
            b.tune(2)
        while b.run(sweeps) > 0:
            pass
        b.run(1)
        for slot in b.finished():
            y, st, hid = b.take(slot)
            out[hid] = (y, st)
    assert len(out) == len(items)
    return out


def test_each_result_is_the_same_alone_and_in_the_mix():
    items = _mix()
    mixed = _run_batch(items)
    for k, it in enumerate(items):
        alone = _run_batch([it])[0]
        np.testing.assert_array_equal(mixed[k][0], alone[0])
        assert mixed[k][1]["steps_acc"] == alone[1]["steps_acc"]
        assert mixed[k][1]["steps_rej"] == alone[1]["steps_rej"]


def test_batch_equals_oracle_bit_for_bit(oracle):
    """Every instance of an uneven mix (BRUSS2D-MIX, LV pairs, banded LV) takes
    the oracle's step counts and ends on its state bit for bit."""
    items = _mix()
    res = _run_batch(items)
    handed = 0
    for k, (p, y0, t0, te, tol) in enumerate(items):
        kind = {rk.PROBLEM_BRUSS2D_MIX: oracle.BRUSS2D_MIX, rk.PROBLEM_LV_PAIRS: oracle.LV_PAIRS,
                rk.PROBLEM_LV_BANDED: oracle.LV_BANDED}[p.kind]
        ref, rst = oracle.solve(kind, y0, "DOPRI54", t0, te, tol, grid_n=p.grid_n, alpha=p.alpha,
                                lv_r=p.lv_r, lv_a=p.lv_a)
        y, st = res[k]
        assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"]), k
        np.testing.assert_array_equal(y, ref)
        handed += st["host_pow_steps"]
    print(f"step-size updates answered by the host: {handed}")


BATCH_GOLDEN = ["bruss_n512_a1e-2_tol1e-8", "bruss_n512_a1e-3_tol1e-4", "bruss_n16_a1e-2_tol1e-8",
                "bruss_n16_a1e-3_tol1e-4", "bruss_n250_dopri54_tol1e-6", "bruss_n100_dopri54_tol1e-6",
                "bruss_n2_dopri54", "bruss_n3_dopri54", "bruss_n4_dopri54", "bruss_n8_dopri54",
                "lv_pairs_1000_dopri54"]


def test_batch_reproduces_reference_goldens():
    """The reference's own results, solved together in one batch: N from 2 to
    512 (the batched configuration's range and the boundary cases), alpha and
    tol across its distribution, and the LV pairs module.  Step counts and the
    final state (sha256 of every component) equal the reference's."""
    recs = [load_golden(n) for n in BATCH_GOLDEN]
    items = []
    for rec in recs:
        p = (rk.bruss2d_mix(rec["grid_n"], rec["alpha"]) if rec["problem"] == "bruss2d-mix"
             else rk.lv_pairs(rec["n"] // 2))
        items.append((p, golden_y0(rec), rec["t0"], rec["t_end"], rec["tol"]))
    res = _run_batch(items, sweeps=256)
    handed = 0
    for k, rec in enumerate(recs):
        y, st = res[k]
        assert (st["steps_acc"], st["steps_rej"]) == (rec["accepted"], rec["rejected"]), rec["name"]
        idx, ref = golden_y(rec)
        np.testing.assert_array_equal(y[idx], ref)
        assert hashlib.sha256(y.astype("<f8").tobytes()).hexdigest() == rec["y_sha256"], rec["name"]
        handed += st["host_pow_steps"]
    assert handed > 0  # the host's pow was needed somewhere, and the results still match


def test_fma_mode_within_tolerance_and_independent_of_the_mix(oracle):
    """FMA mode (products that stay products in software, the rest fused):
    each instance within its tolerance of the oracle, and alone = in the mix."""
    items = _mix(seed=5)[:10] + _mix(seed=5)[18:20]
    res = _run_batch(items, precision="fma")
    for k, (p, y0, t0, te, tol) in enumerate(items):
        kind = {rk.PROBLEM_BRUSS2D_MIX: oracle.BRUSS2D_MIX, rk.PROBLEM_LV_PAIRS: oracle.LV_PAIRS}[p.kind]
        ref, _ = oracle.solve(kind, y0, "DOPRI54", t0, te, tol, grid_n=p.grid_n, alpha=p.alpha)
        y, _ = res[k]
        assert float(np.max(np.abs(y - ref)) / np.max(np.abs(ref))) <= 10 * tol
    alone = _run_batch(items[:1], precision="fma")[0]
    np.testing.assert_array_equal(res[0][0], alone[0])


def test_tuning_and_graph_replay_change_nothing():
    items = _mix(seed=9)[:12]
    a = _run_batch(items, tune=True, graph=True)
    b = _run_batch(items, tune=False, graph=False)
    for k in a:
        np.testing.assert_array_equal(a[k][0], b[k][0])


def test_large_instance_same_under_every_shape():
    """One instance whose pairs (N=256: 65536) are far fewer than two tuned chunks per CTA,
    so the chunk list is built with shortened chunks; every block size and tuned chunk
    length gives the same result."""
    p = rk.bruss2d_mix(256, 2e-3)
    y0 = rk.ode_start(p)
    with rk.Solver(p, method="DOPRI54", precision="exact") as s:
        ref, rst = s.solve(0.0, 0.02, y0, 1e-6)
    results = []
    for threads, chunk in ((128, 256), (256, 1024), (256, 4096), (512, 4096)):
        with rk.Batch(rk.footprint(p, 7) + (64 << 20), 4, precision="exact") as b:
            b.set_tuning(threads, chunk)
            assert b.add(p, y0, 0.0, 0.02, 1e-6, host_id=0) is not None
            while b.run(64) > 0:
                pass
            b.run(1)
            (slot,) = b.finished()
            y, st, _ = b.take(slot)
        results.append((y, st))
    for y, st in results:
        np.testing.assert_array_equal(y, ref)
        assert (st["steps_acc"], st["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])


def test_admission_by_hbm_footprint():
    p = rk.bruss2d_mix(64, 2e-3)
    y0 = rk.ode_start(p)
    fp = rk.footprint(p, 7)
    with rk.Batch(2 * fp, 16) as b:
        s1 = b.add(p, y0, 0.0, 0.01, 1e-6)
        s2 = b.add(p, y0, 0.0, 0.01, 1e-6)
        assert s1 is not None and s2 is not None
        assert b.add(p, y0, 0.0, 0.01, 1e-6) is None        # does not fit: refused
        assert b.info()["free_bytes"] < fp
        while b.run(32) > 0:
            pass
        done = b.finished()
        assert sorted(done) == sorted([s1, s2])
        y, st, _ = b.take(done[0])
        assert b.add(p, y0, 0.0, 0.01, 1e-6) is not None    # admitted after space was freed


def test_batched_workload_sample_matches_plain_form():
    """A seeded sample of the batched configuration's instance distribution (smaller N
    to keep the test short): batch results equal the plain exact path bit for bit."""
    insts = workloads.batched_instances(24, seed=11, n_min=16, n_max=64)
    items = []
    for d in insts:
        p = rk.bruss2d_mix(d["grid_n"], d["alpha"])
        items.append((p, rk.ode_start(p), d["t0"], d["te"], d["tol"]))
    res = _run_batch(items)
    for k, (p, y0, t0, te, tol) in enumerate(items):
        with rk.Solver(p, method="DOPRI54", precision="exact") as s:
            ref, rst = s.solve(t0, te, y0, tol)
        np.testing.assert_array_equal(res[k][0], ref)
        assert (res[k][1]["steps_acc"], res[k][1]["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])

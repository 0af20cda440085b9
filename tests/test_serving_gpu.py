"""Continuous-batching serving loop: requests arriving over time share the GPU,
are admitted by HBM footprint as space frees up, and each result is the same
as when the request is solved alone."""
import numpy as np
import pytest

import rk_gb300 as rk
from rk_gb300.serving import ServingLoop, make_request_problem

pytestmark = pytest.mark.gpu


def _requests(count=36, seed=4):
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for k in range(count):
        t += rng.exponential(0.0005)
        if k % 2 == 0:
            out.append(dict(kind="bruss", arrival=t, grid_n=int(rng.integers(8, 48)), alpha=2e-3,
                            tol=1e-6, t0=0.0, te=0.5))
        else:
            out.append(dict(kind="lv", arrival=t, n=int(rng.integers(100, 5000)),
                            lv_seed=int(rng.integers(1 << 30)), tol=1e-6, t0=0.0, te=10.0))
    return out


def test_serving_admits_by_footprint_and_matches_solo_results():
    reqs = _requests()
    fps = [rk.footprint(make_request_problem(r)[0], 7) for r in reqs]
    arena = int(sum(sorted(fps)[-2:]))          # room for about two of the largest at once
    loop = ServingLoop(arena, max_instances=64)      # launches as time slices
    try:
        out = loop.serve(reqs, keep_results=True)
    finally:
        loop.close()
    assert len(out["results"]) == len(reqs)
    assert out["refusals"] > 0                  # some requests had to wait for memory
    # continuous batching: some request was admitted while another was still running
    adm, fin = out["admitted"], out["finish"]
    assert any(adm[j] < fin[i] and adm[j] > adm[i] for i in range(len(reqs)) for j in range(len(reqs)))
    assert np.all(out["latency"] > 0)
    # each result equals the same request served alone
    for i in (0, 1, 7, 20, 35):
        solo = ServingLoop(1 << 30, max_instances=4, sweeps_per_launch=8)
        try:
            one = solo.serve([dict(reqs[i], arrival=0.0)], keep_results=True)
        finally:
            solo.close()
        y_mix, st_mix = out["results"][i]
        y_solo, st_solo = one["results"][0]
        np.testing.assert_array_equal(y_mix, y_solo)
        assert (st_mix["steps_acc"], st_mix["steps_rej"]) == (st_solo["steps_acc"], st_solo["steps_rej"])
        # and equal to the plain exact path (the reference's arithmetic) bit for bit
        p, y0, t0, te, tol = make_request_problem(reqs[i])
        with rk.Solver(p, method="DOPRI54", precision="exact") as s:
            ref, rst = s.solve(t0, te, y0, tol)
        np.testing.assert_array_equal(y_mix, ref)
        assert (st_mix["steps_acc"], st_mix["steps_rej"]) == (rst["steps_acc"], rst["steps_rej"])

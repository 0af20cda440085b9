"""The seeded synthetic workloads (rk_gb300/workloads.py, rk_gb300.lv_banded_random)
have the shapes of the batched and served configurations: ranges, log-uniform
sizes, the 50/50 request mix, Poisson arrivals, the banded LV chain's structure,
and the same lists from the same seeds."""
import math

import numpy as np

import rk_gb300 as rk
from rk_gb300 import workloads


def test_batched_instances_distribution():
    inst = workloads.batched_instances()
    assert len(inst) == 4096
    N = np.array([d["grid_n"] for d in inst])
    alpha = np.array([d["alpha"] for d in inst])
    tol = np.array([d["tol"] for d in inst])
    assert N.min() >= 16 and N.max() <= 512
    assert alpha.min() >= 1e-3 and alpha.max() <= 1e-2
    assert tol.min() >= 1e-8 and tol.max() <= 1e-4
    assert all(d["t0"] == 0.0 and d["te"] == 0.5 for d in inst)
    # log-uniform: ln N and ln tol centred on their ranges' midpoints
    assert abs(np.median(np.log(N)) - 0.5 * (math.log(16) + math.log(512))) < 0.1
    assert abs(np.median(np.log(tol)) - 0.5 * (math.log(1e-8) + math.log(1e-4))) < 0.2
    assert abs(np.median(alpha) - 5.5e-3) < 4e-4
    assert workloads.batched_instances() == inst                      # the seed fixes the list
    assert workloads.batched_instances(seed=2025) != inst


def test_served_requests_distribution():
    reqs = workloads.served_requests()
    assert len(reqs) == 20000
    kinds = [r["kind"] for r in reqs]
    assert kinds.count("bruss") == 10000 and kinds.count("lv") == 10000
    t = np.array([r["arrival"] for r in reqs])
    gaps = np.diff(t)
    assert np.all(gaps >= 0) and t[0] > 0
    assert abs(gaps.mean() - 1.0 / 100.0) < 0.05 / 100.0               # Poisson, 100 per second
    assert abs(np.std(gaps) / np.mean(gaps) - 1.0) < 0.05               # exponential gaps
    bN = np.array([r["grid_n"] for r in reqs if r["kind"] == "bruss"])
    ln = np.array([r["n"] for r in reqs if r["kind"] == "lv"])
    assert bN.min() >= 32 and bN.max() <= 1024
    assert ln.min() >= 1000 and ln.max() <= 1000000
    assert abs(np.median(np.log(bN)) - 0.5 * (math.log(32) + math.log(1024))) < 0.1
    assert abs(np.median(np.log(ln)) - 0.5 * (math.log(1e3) + math.log(1e6))) < 0.15
    for r in reqs[:200]:
        assert r["tol"] == 1e-6 and r["t0"] == 0.0
        assert r["te"] == (0.5 if r["kind"] == "bruss" else 10.0)
    assert workloads.served_requests() == reqs


def test_banded_lv_instance_structure():
    n = 1000
    p, y0 = rk.lv_banded_random(n, seed=11)
    r, a = p.lv_r, p.lv_a
    assert p.n == n and a.shape == (n, 5)
    assert np.all((r >= 0.5) & (r <= 1.5)) and np.all((y0 >= 0.5) & (y0 <= 1.5))
    assert np.all(a[:, 2] == -1.0)                                      # a_ii
    off = np.delete(a, 2, axis=1)
    assert np.all(np.abs(off) <= 0.1)
    # a[i, k] couples y_i to y_(i + k - 2): the band is cut at both ends
    assert a[0, 0] == a[0, 1] == a[1, 0] == 0.0
    assert a[n - 1, 3] == a[n - 1, 4] == a[n - 2, 4] == 0.0
    assert np.count_nonzero(off[2:n - 2]) == off[2:n - 2].size
    p2, y2 = rk.lv_banded_random(n, seed=11)
    assert np.array_equal(p2.lv_a, a) and np.array_equal(y2, y0)

"""Seeded synthetic workloads with the shapes of the batched and served configurations.

batched_instances: BRUSS2D-MIX instances, N = round(exp(U[ln 16, ln 512])),
    alpha ~ U[1e-3, 1e-2], tol = exp(U[ln 1e-8, ln 1e-4]), t in [0, 0.5] (DOPRI5(4)).
served_requests: a Poisson arrival stream, half BRUSS2D-MIX (N log-uniform in
    [32, 1024], t in [0, 0.5]) and half banded Lotka-Volterra chains (n
    log-uniform in [1e3, 1e6], r ~ U[0.5, 1.5], a_ii = -1, a_ij ~ U[-0.1, 0.1]
    for 0 < |i-j| <= 2, y0 ~ U[0.5, 1.5], t in [0, 10]), tol 1e-6.
"""
import math

import numpy as np


def batched_instances(count=4096, seed=2024, n_min=16, n_max=512):
    rng = np.random.default_rng(seed)
    N = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), count))).astype(int)
    alpha = rng.uniform(1e-3, 1e-2, count)
    tol = np.exp(rng.uniform(math.log(1e-8), math.log(1e-4), count))
    return [dict(grid_n=int(n), alpha=float(a), tol=float(t), t0=0.0, te=0.5)
            for n, a, t in zip(N, alpha, tol)]


def estimated_work(inst):
    """Component-steps of a BRUSS instance: about 1.2 alpha (N-1)^2 attempted steps of
    2 N^2 components when the step size is stability-limited (DOPRI5(4), t in [0, 0.5])."""
    N = inst["grid_n"]
    steps = max(20.0, 1.2 * inst["alpha"] * (N - 1) ** 2)
    return 2.0 * N * N * steps


def served_requests(count=20000, seed=7, rate_per_s=100.0):
    """List of dicts: arrival time (s, Poisson process of the given rate), kind,
    and the parameters of the request; banded LV data are generated on demand
    from the request's own seed (lv_seed)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, count)
    arrival = np.cumsum(gaps)
    kinds = np.array(["bruss"] * (count // 2) + ["lv"] * (count - count // 2))
    rng.shuffle(kinds)
    out = []
    for k, t in zip(kinds, arrival):
        if k == "bruss":
            N = int(round(math.exp(rng.uniform(math.log(32), math.log(1024)))))
            out.append(dict(kind="bruss", arrival=float(t), grid_n=N, alpha=2e-3, tol=1e-6,
                            t0=0.0, te=0.5))
        else:
            n = int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e6)))))
            out.append(dict(kind="lv", arrival=float(t), n=n, lv_seed=int(rng.integers(1 << 31)),
                            tol=1e-6, t0=0.0, te=10.0))
    return out

"""Continuous-batching request loop over the batched step loop (rk_gb300.Batch).

Requests arrive over time (a Poisson stream in the benchmark).  Each arrived
request waits in a queue until its device footprint fits in the arena
(admission by HBM footprint) and a slot is free; then it joins the running
batch, whose persistent kernel advances every admitted solve by a few sweeps
per launch.  Requests that arrive while others are on the GPU are admitted
between launches as slots and memory free up, so their work overlaps on the
device; finished solves are copied out and their space reused at once.
The launches are time slices: the sweep count of the next launch is chosen
from the measured time per sweep so that a launch lasts about `slice_s`,
which bounds how long an arriving request waits for admission while the
sweeps stay long enough to keep the GPU busy.
Latency of a request = completion time - arrival time.
"""
import time

import numpy as np

import rk_gb300 as rk


def make_request_problem(req):
    """(problem, y0, t0, te, tol) of a request dict from rk_gb300.workloads.served_requests."""
    if req["kind"] == "bruss":
        p = rk.bruss2d_mix(req["grid_n"], req.get("alpha", 2e-3))
        return p, rk.ode_start(p), req["t0"], req["te"], req["tol"]
    p, y0 = rk.lv_banded_random(req["n"], seed=req["lv_seed"])
    return p, y0, req["t0"], req["te"], req["tol"]


class ServingLoop:
    """sweeps_per_launch > 0 fixes the sweeps per launch; 0 chooses them per
    launch as a time slice of about slice_s (a power of two, 1 .. max_sweeps).
    `batch` serves through an existing object with rk_gb300.Batch's add / run /
    finished / take / tune methods instead of a new Batch."""

    def __init__(self, arena_bytes, max_instances=4096, sweeps_per_launch=0, precision="exact",
                 method="DOPRI54", device=0, stream=None, slice_s=0.004, max_sweeps=64, batch=None):
        self.batch = batch if batch is not None else rk.Batch(
            arena_bytes, max_instances, method=method, precision=precision, device=device, stream=stream)
        self.fixed = sweeps_per_launch
        self.sweeps = sweeps_per_launch if sweeps_per_launch > 0 else 4
        self.slice_s = slice_s
        self.max_sweeps = max_sweeps
        self.sweep_s = None               # running estimate of one sweep's time

    def _run_slice(self):
        """One launch; updates the per-sweep time estimate and the next sweep count."""
        t = time.perf_counter()
        active = self.batch.run(self.sweeps)
        dt = (time.perf_counter() - t) / self.sweeps
        if not self.fixed:
            self.sweep_s = dt if self.sweep_s is None else 0.7 * self.sweep_s + 0.3 * dt
            want = max(1.0, self.slice_s / max(self.sweep_s, 1e-7))
            self.sweeps = int(min(self.max_sweeps, 2 ** int(np.floor(np.log2(want)))))
        return active

    def close(self):
        self.batch.close()

    def serve(self, requests, time_scale=1.0, keep_results=False, make=make_request_problem,
              tune_after=0):
        """Serve `requests` (dicts with an "arrival" time in seconds, sorted) in real
        time scaled by time_scale.  Returns a dict with per-request latencies,
        completion times, the number of admission refusals, throughput and, if
        keep_results, every result (y, stats) by request index."""
        n = len(requests)
        arrival = np.array([r["arrival"] for r in requests]) * time_scale
        queue = []                        # indices of arrived, not yet admitted requests
        payload = {}                      # index -> (problem, y0, t0, te, tol)
        finish = np.full(n, np.nan)
        admitted_at = np.full(n, np.nan)
        results = {}
        refusals = 0
        nxt = 0
        active = 0
        done = 0
        tuned = tune_after <= 0
        t_start = time.perf_counter()
        while done < n:
            now = time.perf_counter() - t_start
            while nxt < n and arrival[nxt] <= now:
                queue.append(nxt)
                nxt += 1
            # admission: every queued request whose footprint fits, in arrival order
            still = []
            for i in queue:
                if i not in payload:
                    payload[i] = make(requests[i])
                p, y0, t0, te, tol = payload[i]
                slot = self.batch.add(p, y0, t0, te, tol, host_id=i)
                if slot is None:
                    refusals += 1
                    still.append(i)
                else:
                    admitted_at[i] = time.perf_counter() - t_start
                    active += 1
            queue = still
            if active == 0:
                if nxt < n:  # idle until the next arrival
                    time.sleep(max(0.0, min(arrival[nxt] - (time.perf_counter() - t_start), 0.05)))
                continue
            if not tuned and active >= tune_after:
                self.batch.tune(1)
                tuned = True
            active = self._run_slice()
            for slot in self.batch.finished():
                y, st, i = self.batch.take(slot)
                finish[i] = time.perf_counter() - t_start
                payload.pop(i, None)
                done += 1
                if keep_results:
                    results[i] = (y, st)
        makespan = time.perf_counter() - t_start
        lat = finish - arrival
        return dict(latency=lat, finish=finish, admitted=admitted_at, refusals=refusals,
                    makespan=makespan, solves_per_s=n / makespan,
                    p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)),
                    results=results)


def serve_plain(requests, time_scale=1.0, precision="exact", make=make_request_problem):
    """The plain form as a server: one request at a time, first come first served."""
    n = len(requests)
    arrival = np.array([r["arrival"] for r in requests]) * time_scale
    finish = np.full(n, np.nan)
    t_start = time.perf_counter()
    for i, req in enumerate(requests):
        now = time.perf_counter() - t_start
        if arrival[i] > now:
            time.sleep(arrival[i] - now)
        p, y0, t0, te, tol = make(req)
        with rk.Solver(p, method="DOPRI54", precision=precision) as s:
            s.solve(t0, te, y0, tol)
        finish[i] = time.perf_counter() - t_start
    makespan = time.perf_counter() - t_start
    lat = finish - arrival
    return dict(latency=lat, makespan=makespan, solves_per_s=n / makespan,
                p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)))

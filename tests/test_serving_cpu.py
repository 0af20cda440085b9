"""Host logic of the continuous-batching loop (rk_gb300/serving.py) on the CPU,
over a stand-in for the device batch: admission by footprint in arrival order
without head-of-line blocking, every request completed exactly once with its
own result, latency = completion - arrival, the time-slice rule for the sweeps
per launch, and the autotuner started once.  The GPU tests run the same loop
over rk_gb300.Batch."""
import time

import numpy as np

from rk_gb300.serving import ServingLoop


class FakeBatch:
    """Instances advance one step per sweep; a sweep takes sweep_s seconds of
    host time; the arena holds `capacity` bytes of footprints."""

    def __init__(self, capacity, sweep_s=0.0005):
        self.capacity, self.used, self.sweep_s = capacity, 0, sweep_s
        self.slots, self.next_slot, self.done = {}, 0, []
        self.runs, self.tuned, self.admitted = [], 0, []

    def add(self, problem, y0, t0, te, tol, host_id=-1):
        need = problem["bytes"]
        if self.used + need > self.capacity:
            return None
        slot = self.next_slot
        self.next_slot += 1
        self.slots[slot] = dict(left=problem["steps"], need=need, host_id=host_id, y=y0.copy(),
                                steps=problem["steps"])
        self.used += need
        self.admitted.append(host_id)
        return slot

    def run(self, sweeps):
        self.runs.append(sweeps)
        time.sleep(self.sweep_s * sweeps)
        active = 0
        for slot, d in self.slots.items():
            if d["left"] > 0:
                d["left"] -= sweeps
                d["y"] += 1.0
                if d["left"] <= 0:
                    self.done.append(slot)
                else:
                    active += 1
        return active

    def finished(self):
        out, self.done = self.done, []
        return out

    def take(self, slot):
        d = self.slots.pop(slot)
        self.used -= d["need"]
        return d["y"], {"steps": d["steps"]}, d["host_id"]

    def tune(self, sweeps_per_trial=2):
        self.tuned += 1


def make(req):
    return dict(steps=req["steps"], bytes=req["bytes"]), np.full(4, float(req["id"])), 0.0, 1.0, 1e-6


def requests(n, seed=3, big_every=0):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(0.002, n))
    out = []
    for i in range(n):
        big = big_every and i % big_every == 0
        out.append(dict(id=i, arrival=float(t[i]), steps=int(rng.integers(3, 40)),
                        bytes=800 if big else 100))
    return out


def test_every_request_served_once_with_its_result():
    reqs = requests(60)
    fb = FakeBatch(capacity=1000)
    loop = ServingLoop(0, batch=fb)
    out = loop.serve(reqs, keep_results=True, make=make)
    assert sorted(out["results"]) == list(range(60))
    for i, (y, st) in out["results"].items():
        assert st["steps"] == reqs[i]["steps"]
        assert np.all(y > i)  # its own state, advanced
    assert np.all(np.isfinite(out["latency"])) and np.all(out["latency"] >= 0)
    np.testing.assert_allclose(out["latency"], out["finish"] - np.array([r["arrival"] for r in reqs]))
    assert np.all(out["admitted"] >= np.array([r["arrival"] for r in reqs]) - 1e-9)
    assert sorted(fb.admitted) == list(range(60)) and fb.used == 0


def test_admission_by_footprint_without_head_of_line_blocking():
    # a large request that does not fit waits; smaller ones behind it are admitted
    reqs = [dict(id=0, arrival=0.0, steps=400, bytes=600), dict(id=1, arrival=0.0, steps=5, bytes=600),
            dict(id=2, arrival=0.0, steps=5, bytes=100), dict(id=3, arrival=0.0, steps=5, bytes=100)]
    fb = FakeBatch(capacity=1000)
    out = ServingLoop(0, batch=fb).serve(reqs, make=make)
    assert fb.admitted[:3] == [0, 2, 3]  # request 1 waits for room, 2 and 3 pass it
    assert out["refusals"] >= 1
    assert out["finish"][2] < out["finish"][1] and out["finish"][3] < out["finish"][1]


def test_time_slices_choose_a_power_of_two():
    reqs = [dict(id=i, arrival=0.0, steps=200, bytes=10) for i in range(4)]
    fb = FakeBatch(capacity=1000, sweep_s=0.001)
    loop = ServingLoop(0, batch=fb, slice_s=0.004, max_sweeps=64)
    loop.serve(reqs, make=make)
    assert all(r & (r - 1) == 0 for r in fb.runs)  # powers of two
    assert max(fb.runs[3:]) <= 4                    # at most 4 ms of sweeps of 1 ms or more
    want = max(1.0, loop.slice_s / loop.sweep_s)    # the rule, from the loop's own estimate
    assert loop.sweeps == min(64, 2 ** int(np.floor(np.log2(want))))
    fb2 = FakeBatch(capacity=1000, sweep_s=0.0001)
    ServingLoop(0, batch=fb2, slice_s=0.004, max_sweeps=8).serve(reqs, make=make)
    assert max(fb2.runs) == 8                       # capped by max_sweeps
    fb3 = FakeBatch(capacity=1000)
    ServingLoop(0, batch=fb3, sweeps_per_launch=3).serve(reqs, make=make)
    assert set(fb3.runs) == {3}                     # a fixed sweep count stays fixed


def test_autotuner_started_once():
    reqs = requests(30, seed=5)
    fb = FakeBatch(capacity=10000)
    ServingLoop(0, batch=fb).serve(reqs, make=make, tune_after=4)
    assert fb.tuned == 1

#!/usr/bin/env python3
"""Benchmark of the embedded-RK step loop on BRUSS2D-MIX (steps/s and %HBM).

Workload: BRUSS2D-MIX on an N=2000 grid (n = 8,000,000 components), DOPRI5(4),
tol 1e-6, t in [0, 0.5], alpha 2e-3, initial values of the problem module --
the FP64 configuration the reference's solver is quoted on.  A "step" is one
attempted RK step (accepted or rejected) over all n components.

  value    steps/s with y resident in HBM, K steps timed with CUDA events on the
           solver's stream (one persistent launch runs the K steps)
  e2e      the same through the C ABI with host buffers: pinned y0 copied in,
           K steps, y copied out, timed on the host clock
  roofline algorithmic bytes (16 n per attempted step: read y, write y) over the
           launch time, against the measured HBM copy bandwidth; the FP64
           pipe, not HBM, bounds this kernel, so "fp64" reports its share too
  cpu_baseline the oracle port (the reference's step loop restated in C in its
           fastest form, the low-storage pipelined schedule of PipeD4ls, pthreads
           over every host core) on a bounded sample of the same steps

--gpus N runs N independent replicas (the path does not shard); value is
the sum over replicas (N K steps over the slowest replica's time).
--impl reference times the reference's CPU algorithm (the oracle port in the
schedule of its fastest pthreads variant, every host thread) on the same
workload instead.
"""
import argparse
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

GRID_N = 2000
ALPHA = 2e-3
TOL = 1e-6
T0, TE = 0.0, 0.5
L2_BYTES = 129e6
FALLBACK_HBM_GBS = 6800.0
# FP64 pipe throughput measured on this GB300 pool with independent DFMA
# chains: 505 G instr/s (1.01 TFLOP/s counting an FMA as 2 flops).
FP64_GOPS_MEASURED = 505.0
# FP64 pipe peak of this part: 2 FP64 instructions per SM per clock.
FP64_PER_SM_CLK = 2.0


# DRAM bytes per component-step of the step-loop kernel, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) at N=2000, DOPRI5(4); all
# vectors exceed L2 at that size and above, so the figure scales with n.
MEASURED_TRAFFIC = {
    ("d", "exact", "DOPRI54"): (584.0, "one-pass ncu capture (dram bytes and duration) of every plain_kernel launch "
                                        "of this benchmark's default headline command: 583.9 B over the 20 timed steps"),
    ("d", "fma", "DOPRI54"): (573.0, "ncu --set full of a 3-step launch at N=2000"),
    ("d", "mixed", "DOPRI54"): (46.9, "ncu --set full of a 3-step launch at N=2000 (fused FP32 stages), scaled by n"),
}

KERNEL_NAME = {"d": "plain_kernel (persistent, all stages of K steps)",
               "lowstorage": "ls_kernel (persistent wavefront, K steps)",
               "mixed": "mixed_kernel (persistent, all stages of K steps)"}


def fp64_ops_per_comp(method, precision):
    """(FP64-pipe instructions, FP64 operations) per component-step of the
    BRUSS2D-MIX step loop, counted from the kernel.  Operations: a right-hand
    side costs 9.5 (exact: 6.5 sums + 3 products) / 7.5 (fused) per component,
    each nonzero tableau coefficient a product and a sum (exact) or one FMA,
    the update one sum, the error norm one division per thread and step (its
    maximum is kept as an undivided quotient).  On the FP64
    pipe: the Laplacian's four sums run on the integer pipe (exact integer
    arithmetic where the five values share a binade, which is nearly every
    point), so a right-hand side keeps 2.5 sums per component; in the exact
    mode its 3 products per component run on the FP64 pipe (with max/compare
    work 6.3 per right-hand side) while the tableau products run in software
    binary64 on the integer pipe; the fused mode keeps 3.3 per right-hand side
    and computes the first stage's two plain products in software (ncu: 53.7
    FP64-pipe instructions per DOPRI5(4) component-step; exact: DADD 50.6,
    DMUL 21.1, DFMA 0.4, 72.1 in all, plus compares).
    The mixed form evaluates F0 in double-float arithmetic (FP32 pairs, the
    Laplacian in integer fixed point) and keeps three FP64 sums per
    component-step: y + (h sum b F0) as two sums, and y1 + dY."""
    if precision == "mixed":
        return 3.0, 3.0
    import rk_gb300 as rk
    m = rk.builtin_method(method)
    s = m["s"]
    nz_a = int(np.count_nonzero(np.tril(m["A"], -1)))
    nz_b = int(np.count_nonzero(m["b"]))
    nz_bh = int(np.count_nonzero(m["b"] - m["b_hat"]))
    if precision.startswith("exact"):
        ops = 9.5 * s + 2 * nz_a + (2 * nz_b - 1) + (2 * nz_bh - 1) + 1.5
        if precision == "exact-hwmul":
            return 5.5 * s + 2 * nz_a + (2 * nz_b - 1) + (2 * nz_bh - 1) + 1.5, ops
        return 6.3 * s + nz_a + (nz_b - 1) + (nz_bh - 1) + 0.5, ops
    ops = 7.5 * s + nz_a + nz_b + nz_bh + 1.5
    return 3.3 * s + nz_a + (nz_b - 1) + (nz_bh - 1) + 1.5, ops


E2E_RUNS = 3


def _peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        with open(self.tmp.name) as f:
            rows = [r.split(",") for r in f.read().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _init_pg(ws, backend):
    import torch.distributed as dist
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return dist if ws > 1 else None


def _max_over_ranks(x, dist, device=None):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# the CPU port's schedule: the low-storage pipelined one (the reference's
# fastest pthreads variant, PipeD4ls); bit-identical to the D schedule
PORT_SCHEDULE = "low-storage pipelined schedule (PipeD4ls form)"


def port_solve(rk_oracle, y0, tol, steps, threads, grid_n=GRID_N, alpha=ALPHA, t0=None, te=None):
    return rk_oracle.solve(rk_oracle.BRUSS2D_MIX, y0, "DOPRI54", T0 if t0 is None else t0,
                           TE if te is None else te, tol, step_limit=steps, grid_n=grid_n,
                           alpha=alpha, threads=threads, rows=1)


def cpu_baseline_port(threads, target_s=12.0, max_steps=400):
    """Time the oracle port (the reference's step loop in C, pthreads) on the
    full-size problem: as many steps as fit in about target_s, at least 2."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import rk_oracle
    y0 = rk_oracle.bruss_start(GRID_N)
    t = time.perf_counter()
    port_solve(rk_oracle, y0, TOL, 1, threads)
    one = time.perf_counter() - t
    steps = int(max(2, min(max_steps, target_s / max(one, 1e-6))))
    t = time.perf_counter()
    _, st = port_solve(rk_oracle, y0, TOL, steps, threads)
    dt = time.perf_counter() - t
    done = st["steps_acc"] + st["steps_rej"]
    return done / dt, done, dt


REF_VARIANT = "pthreads/PipeD4ls"


def reference_run(steps, threads, grid_n=GRID_N):
    """Run the reference's own pthreads PipeD4ls solver (its fastest variant),
    compiled from its sources with its own flags and the workload's defines,
    for `steps` attempted steps (the STEP_LIMIT define).  Returns (steps done,
    the solver's own "Kernel time" in s), or None without reference sources or
    a C compiler."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import stage_reference
    defines = dict(BRUSS_GRID_SIZE=grid_n, BRUSS_ALPHA="2E-3", METHOD="DOPRI54", TOL="1E-6",
                   T_END="0.5", STEP_LIMIT=int(steps))
    try:
        exe = stage_reference.build_solver(REF_VARIANT, defines,
                                           name=f"pthreads_bruss2d-mix_PipeD4ls_n{grid_n}_l{steps}")
    except Exception:
        return None
    if not exe:
        return None
    out = subprocess.run([exe], env=dict(os.environ, NUM_THREADS=str(threads)), capture_output=True,
                         text=True, check=True).stdout
    import re
    m = re.search(r"Number of steps: (\d+)", out)
    k = re.search(r"Kernel time: ([0-9.eE+-]+) s", out)
    return int(m.group(1)), float(k.group(1))


def cpu_baseline(threads, target_s=10.0, max_steps=400, min_steps=2):
    """The CPU baseline on the full-size problem: the reference's own PipeD4ls
    binary when its sources are here (kind "reference"), else the oracle port in
    the same schedule (kind "port").  As many steps as fit in about target_s.
    Returns (steps/s, steps, seconds, kind, description)."""
    probe = reference_run(5, threads)
    if probe is not None:
        per = probe[1] / max(1, probe[0])
        steps = int(max(min_steps, min(max_steps, target_s / max(per, 1e-6))))
        done, kt = reference_run(steps, threads)
        return done / kt, done, kt, "reference", (
            f"the reference's {REF_VARIANT} solver compiled from its sources (-O3 -g, its "
            f"flags), first {done} steps of the N={GRID_N} solve (STEP_LIMIT={steps}), "
            f"{threads} threads, its own Kernel time")
    v, done, dt = cpu_baseline_port(threads, target_s, max_steps)
    return v, done, dt, "port", (f"first {done} steps of the same N={GRID_N} solve ({dt:.1f} s), "
                                 f"oracle port, {PORT_SCHEDULE}, {threads} pthreads")


def workload_config(grid_n, method, ws):
    """The `config` both arms print: the workload, not the implementation."""
    n = 2 * grid_n * grid_n
    return {"workload": f"bruss2d-mix N={grid_n} n={n} {method} tol=1e-6 t=[0,0.5]",
            "grid_n": grid_n, "alpha": ALPHA, "method": method, "tol": TOL, "t_end": TE,
            "parallelism": f"replicas{ws}",
            "l2": f"working set {(10 if method == 'DOPRI54' else 16) * 8 * n / 1e6:.0f} MB "
                  f"> {L2_BYTES / 1e6:.0f} MB L2, no flush"}


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # warm-up run, then the timed sample: each "step" is one RK step on the full
    # problem, the sample bounded so that the whole run ends within a few minutes
    probe = reference_run(max(1, args.warmup), threads)
    if probe is not None:
        per = probe[1] / max(1, probe[0])
        k = max(2, min(args.steps, int(90.0 / max(per, 1e-6))))
        k, dt = reference_run(k, threads)
        kind, sample = "reference", (f"the reference's {REF_VARIANT} solver compiled from its "
                                     f"sources, first {k} steps of the N={GRID_N} solve, "
                                     f"{threads} threads, its own Kernel time")
    else:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import rk_oracle
        y0 = rk_oracle.bruss_start(GRID_N)
        t = time.perf_counter()
        port_solve(rk_oracle, y0, TOL, max(1, args.warmup), threads)
        per = (time.perf_counter() - t) / max(1, args.warmup)
        k = max(2, min(args.steps, int(90.0 / max(per, 1e-6))))
        t = time.perf_counter()
        _, st = port_solve(rk_oracle, y0, TOL, k, threads)
        dt = time.perf_counter() - t
        k = st["steps_acc"] + st["steps_rej"]
        kind, sample = "port", (f"first {k} steps of the N={GRID_N} solve, oracle port "
                                f"({PORT_SCHEDULE}), {threads} pthreads")
    v = k / dt
    line = {
        "impl": "reference", "metric": f"BRUSS2D-MIX N={GRID_N} DOPRI54 steps/s", "value": v,
        "unit": "steps/s", "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / k, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (ode_start initial values of BRUSS2D-MIX)",
        "config": workload_config(GRID_N, "DOPRI54", ws),
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import ctypes

    import torch

    import rk_gb300 as rk

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = _init_pg(ws, "nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    prob = rk.bruss2d_mix(args.grid, ALPHA)
    n = prob.n
    y0 = rk.ode_start(prob)
    y0_dev = torch.from_numpy(y0).to(dev)
    torch.cuda.synchronize()

    solver = rk.Solver(prob, method=args.method, precision=args.precision, device=local,
                       stream=stream.cuda_stream,
                       variant=rk.VARIANT_LOWSTORAGE if args.variant == "lowstorage" else rk.VARIANT_D,
                       block_rows=args.block_rows, schedule=args.schedule,
                       flow_skew=args.flow_skew)
    # ---- device-resident timing -------------------------------------------
    # (the clock sampler starts before the warm-up, so that starting it leaves
    # no idle gap between the warm-up and the timed steps)
    clocks = ClockSampler(local)
    clocks.start()
    solver.begin(T0, TE, None, TOL, y0_device_ptr=y0_dev.data_ptr())
    st0 = solver.run(args.warmup)
    launches0 = solver.launches
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    st = solver.run(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    clk = clocks.stop()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = solver.launches - launches0
    steps_done = st["steps_acc"] + st["steps_rej"] - (st0["steps_acc"] + st0["steps_rej"])
    host_pow_steps = st["host_pow_steps"] - st0["host_pow_steps"]
    ms = ev0.elapsed_time(ev1)
    ms_max = _max_over_ranks(ms, dist, dev)
    value = ws * steps_done / (ms_max * 1e-3)

    # ---- end to end through the C ABI with host buffers -------------------
    pinned_in = torch.from_numpy(y0).pin_memory()
    pinned_out = torch.empty(n, dtype=torch.float64).pin_memory()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    lib = rk.load()
    # three runs from y0, the median reported: one run is a few tens of ms of
    # host-clock timing, which a host hiccup on the shared machine can stretch
    e2e_runs = []
    for _ in range(E2E_RUNS):
        launches_e0 = solver.launches
        t = time.perf_counter()
        rc = lib.rkcu_begin(solver._h, T0, TE, ctypes.c_void_p(pinned_in.data_ptr()), 0, TOL)
        assert rc == 0, rc
        solver.run(args.steps)
        rc = lib.rkcu_get_y(solver._h, ctypes.c_void_p(pinned_out.data_ptr()), 0)
        assert rc == 0, rc
        e2e_s = time.perf_counter() - t
        st2 = solver.query()
        e2e_steps = st2["steps_acc"] + st2["steps_rej"]
        e2e_s = _max_over_ranks(e2e_s, dist, dev)
        e2e_runs.append((ws * e2e_steps / e2e_s, solver.launches - launches_e0))
    e2e_value = sorted(v for v, _ in e2e_runs)[len(e2e_runs) // 2]
    dev_bytes = solver.device_bytes
    solver.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = _peaks()
    per_step_bytes = 16.0 * n
    launch_s = ms * 1e-3 / max(1, launches)
    achieved = per_step_bytes * steps_done / max(1, launches) / launch_s / 1e9
    opc, alg_opc = fp64_ops_per_comp(args.method, args.precision)
    fp64_ops = opc * n * steps_done
    fp64_achieved = fp64_ops / (ms * 1e-3) / 1e9
    import torch
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    clk_mhz = clk.get("sm_mhz") or 2070.0
    fp64_peak = FP64_PER_SM_CLK * nsm * clk_mhz * 1e6 / 1e9
    tr = MEASURED_TRAFFIC.get((args.variant, args.precision, args.method))
    traffic = tr[0] * n * steps_done / max(1, launches) if tr else None
    kname = KERNEL_NAME["mixed" if args.precision == "mixed" else args.variant]
    line = {
        "metric": f"BRUSS2D-MIX N={args.grid} {args.method} steps/s", "value": value, "unit": "steps/s",
        "n_gpus": ws, "steps": steps_done, "warmup": args.warmup,
        "ms_per_step": ms_max / max(1, steps_done), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision != "mixed" else "f32 stages / f64 state",
        "data": "synthetic (ode_start initial values of BRUSS2D-MIX)",
        "config": workload_config(args.grid, args.method, ws),
        "implementation": {"precision": args.precision, "variant": args.variant,
                           "device_working_set_mb": round(dev_bytes / 1e6)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "traffic_bytes_per_component_step": tr[0] if tr else None,
                     "traffic_source": tr[1] if tr else "not measured for this configuration",
                     "dram_achieved": traffic / launch_s / 1e9 if tr else None,
                     "dram_frac": traffic / launch_s / 1e9 / peak if tr else None,
                     "kernel": kname},
        "fp64_roofline": {"achieved": fp64_achieved, "peak": fp64_peak,
                          "unit": "G FP64 instr/s", "frac": fp64_achieved / fp64_peak,
                          "peak_kind": f"2 FP64 instr/clk/SM x {nsm} SMs at the sampled {clk_mhz:.0f} MHz "
                                       f"(a DFMA-chain probe reaches {FP64_GOPS_MEASURED:.0f} G/s)",
                          "frac_of_probe": fp64_achieved / FP64_GOPS_MEASURED,
                          "fp64_instr_per_component_step": opc,
                          "fp64_ops_per_component_step": alg_opc},
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": 8.0 * n / max(1, e2e_steps),
                "d2h_bytes_per_step": 8.0 * n / max(1, e2e_steps),
                "runs": [round(v, 1) for v, _ in e2e_runs], "launches_per_run": [l for _, l in e2e_runs],
                "note": f"C-ABI begin/advance/get_y of {e2e_steps} steps from y0 with pinned host y0 and y, "
                        f"the median of {E2E_RUNS} runs"},
        "gpu_launches": launches,
        "host_pow_steps": host_pow_steps,
        "clocks": clk,
        "device_bytes": dev_bytes,
    }
    if args.precision == "mixed":
        line["error_vs_fp64"] = mixed_error_vs_fp64(rk, prob, y0, args.method)
    if not args.no_cpu_baseline and args.grid == GRID_N and args.method == "DOPRI54":
        threads = os.cpu_count() or 1
        v, k, dt, kind, sample = cpu_baseline(threads)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": threads, "kind": kind,
                                "sample": sample}
    if ws == 1 and not args.no_forms and args.grid == GRID_N and args.method == "DOPRI54":
        # the metric's second half: batched solves/s, served p50/p99 against the
        # plain form, and the mixed-precision configuration, each timed on its own
        line["mixed"] = form_mixed(rk, local, peak, peak_kind)
        line["batched"] = form_batched(rk, args.batched_sample, not args.no_cpu_baseline)
        cap = line["batched"]["component_steps_per_s"]
        line["served"] = [form_served(rk, args.served_requests, load, cap) for load in (0.5, 0.9, 1.5)]
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def form_mixed(rk, device, peak, peak_kind):
    """The mixed-precision configuration, whole: BRUSS2D-MIX N=4000 (n = 3.2e7),
    DOPRI5(4), tol 1e-6, t in [0, 0.5], through the C ABI with host buffers
    (pinned y0 in, y out).  value: attempted steps over the device time of the
    step loop (CUDA events on the solver's stream); e2e: the same steps over
    the host time of begin + steps + get_y.  The error is measured against the
    exact FP64 form's final state (bit-identical to the reference wherever
    compared) at the fixture's stored components."""
    import torch
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    from make_n4000_fixture import sample_indices
    base = os.path.join(REPO, "tests", "golden", "n4000", "bruss_n4000_dopri54_tol1e-6")
    with open(base + ".json") as f:
        rec = json.load(f)
    ref = np.load(base + "_sample.npy")
    idx = sample_indices(rec["grid_n"])
    prob = rk.bruss2d_mix(rec["grid_n"], rec["alpha"])
    n = prob.n
    y0 = torch.from_numpy(rk.ode_start(prob)).pin_memory()
    y = torch.empty(n, dtype=torch.float64).pin_memory()
    stream = torch.cuda.Stream(device=device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with rk.Solver(prob, method="DOPRI54", precision="mixed", device=device,
                   stream=stream.cuda_stream) as s:
        lib = rk.load()
        torch.cuda.synchronize()
        clocks = ClockSampler(device)
        clocks.start()
        t = time.perf_counter()
        import ctypes
        assert lib.rkcu_begin(s._h, rec["t0"], rec["t_end"], ctypes.c_void_p(y0.data_ptr()), 0,
                              rec["tol"]) == 0
        ev0.record(stream)
        st = s.run(1 << 30)
        ev1.record(stream)
        assert lib.rkcu_get_y(s._h, ctypes.c_void_p(y.data_ptr()), 0) == 0
        e2e_s = time.perf_counter() - t
        ev1.synchronize()
        clk = clocks.stop()
        launches = s.launches
    ms = ev0.elapsed_time(ev1)
    steps = st["steps_acc"] + st["steps_rej"]
    yv = y.numpy()
    err = float(np.max(np.abs(yv[idx] - ref)) / np.max(np.abs(ref)))
    achieved = 16.0 * n * steps / (ms * 1e-3) / 1e9
    tr = MEASURED_TRAFFIC.get(("d", "mixed", "DOPRI54"))
    return {
        "metric": "mixed-precision BRUSS2D-MIX N=4000 steps/s", "value": steps / (ms * 1e-3),
        "unit": "steps/s", "steps": steps, "accepted": st["steps_acc"], "rejected": st["steps_rej"],
        "ms_per_step": ms / steps, "dtype": "f32 stages / f64 state", "gpu_launches": launches,
        "config": {"workload": f"bruss2d-mix N={rec['grid_n']} n={n} DOPRI54 tol=1e-6 t=[0,0.5], "
                               "the whole solve", "l2": "2 x 256 MB FP64 state + 3 x 128 MB FP32 "
                               "vectors > 129 MB L2, no flush"},
        "e2e": {"value": steps / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": 8.0 * n / steps,
                "d2h_bytes_per_step": 8.0 * n / steps},
        "error_vs_fp64": {"t_end": rec["t_end"], "rel_max_norm_on_sample": err,
                          "sample": f"{idx.size} components (grid rows 0 and {rec['grid_n'] - 1}, "
                                    "every 977th component)",
                          "fp64_steps": rec["steps"], "tol": rec["tol"], "within_tol": err <= rec["tol"],
                          "rel_max_norm_all_components_when_fixture_was_made":
                              rec["mixed"]["rel_max_norm_full"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": tr[0] * n * steps / max(1, launches) if tr else None,
                     "traffic_bytes_per_component_step": tr[0] if tr else None,
                     "traffic_source": tr[1] if tr else None,
                     "dram_frac": tr[0] * n * steps / (ms * 1e-3) / 1e9 / peak if tr else None,
                     "kernel": "mixed_kernel (persistent; stage 0, then all FP32 stages per tile)"},
        "clocks": clk,
    }


def form_batched(rk, count, cpu):
    """Batched configuration on a seeded sample of its 4096-instance list (N
    log-uniform [16,512], alpha U[1e-3,1e-2], tol log-uniform [1e-8,1e-4],
    DOPRI5(4), t in [0, 0.5]): one batch, solves/s on the device (CUDA events
    from the first sweep to the last), e2e with the admissions (host y0 copies)
    and the result copies; the plain form and the CPU port solving the SAME
    instances one after another (plain) and one per host thread (CPU)."""
    import concurrent.futures as cf

    import torch

    from rk_gb300 import workloads

    insts = workloads.batched_instances(4096, seed=2024)
    rng = np.random.default_rng(5)
    pick = sorted(rng.choice(len(insts), count, replace=False))
    sample = [insts[i] for i in pick]
    probs = [rk.bruss2d_mix(d["grid_n"], d["alpha"]) for d in sample]
    y0s = [rk.ode_start(p) for p in probs]
    arena = sum(rk.footprint(p, 7) for p in probs) + (64 << 20)
    clocks = ClockSampler(0)
    clocks.start()
    with rk.Batch(arena, len(sample) + 1, precision="exact") as b:
        t_e2e = time.perf_counter()
        for k, (p, y0, d) in enumerate(zip(probs, y0s, sample)):
            assert b.add(p, y0, d["t0"], d["te"], d["tol"], host_id=k) is not None
        stream = torch.cuda.ExternalStream(b.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        sweeps = 0
        while b.run(256) > 0:
            sweeps += 256
        ev1.record(stream)
        ev1.synchronize()
        results = {}
        for slot in b.finished():
            y, st, hid = b.take(slot)
            results[hid] = (y, st)
        e2e_s = time.perf_counter() - t_e2e
        info = b.info()
        tuning = b.tuning()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    comp_steps = sum(p.n * (results[k][1]["steps_acc"] + results[k][1]["steps_rej"])
                     for k, p in enumerate(probs))
    host_pow = sum(results[k][1]["host_pow_steps"] for k in results)
    # the plain form on the same instances, one after another
    t = time.perf_counter()
    same = 0
    for k, (p, y0, d) in enumerate(zip(probs, y0s, sample)):
        with rk.Solver(p, method="DOPRI54", precision="exact") as s:
            y, st = s.solve(d["t0"], d["te"], y0, d["tol"])
        same += int(np.array_equal(y, results[k][0]))
    plain_s = time.perf_counter() - t
    out = {
        "metric": "batched BRUSS2D-MIX solves/s", "value": len(sample) / (ms * 1e-3),
        "unit": "solves/s", "instances": len(sample), "sweeps": sweeps, "dtype": "f64",
        "config": {"workload": f"batched: {len(sample)} of the 4096 seeded instances (seed 2024, "
                               f"sample seed 5), {100.0 * len(sample) / 4096:.1f} % of the list",
                   "tuning": tuning},
        "component_steps_per_s": comp_steps / (ms * 1e-3),
        "e2e": {"value": len(sample) / e2e_s, "unit": "solves/s",
                "h2d_bytes_per_step": sum(8 * p.n for p in probs) / max(1, sweeps),
                "d2h_bytes_per_step": sum(8 * p.n for p in probs) / max(1, sweeps)},
        "plain_form": {"value": len(sample) / plain_s, "unit": "solves/s",
                       "sample": "the same instances, one solve after another (host buffers)",
                       "results_bit_identical_to_batch": same},
        "host_pow_steps": host_pow, "gpu_launches": info["launches"], "clocks": clk,
    }
    if cpu:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import rk_oracle
        rk_oracle.load()
        threads = os.cpu_count() or 1

        def one(k):
            d = sample[k]
            return port_solve(rk_oracle, y0s[k], d["tol"], 0, 1, grid_n=d["grid_n"],
                              alpha=d["alpha"], t0=d["t0"], te=d["te"])
        t = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            outs = list(ex.map(one, range(len(sample))))
        cpu_s = time.perf_counter() - t
        same = sum(int(np.array_equal(o[0], results[k][0])) for k, o in enumerate(outs))
        out["cpu_baseline"] = {"value": len(sample) / cpu_s, "unit": "solves/s", "cores": threads,
                               "kind": "port",
                               "sample": f"the same {len(sample)} instances, one per host thread "
                                         f"({cpu_s:.1f} s); the reference fixes N and alpha at "
                                         "compile time, so its oracle port solves them",
                               "results_bit_identical_to_batch": same}
    return out


def form_served(rk, count, load, capacity):
    """Served configuration on the first `count` requests of the seeded
    20,000-request Poisson stream, arrivals rescaled so that the offered work
    is `load` times the batched capacity just measured; the plain form serves
    the same requests with the same arrivals, one at a time."""
    from rk_gb300 import serving, workloads
    reqs = workloads.served_requests(20000, seed=7)[:count]
    work = 0.0
    for r in reqs:
        if r["kind"] == "bruss":
            work += workloads.estimated_work(dict(grid_n=r["grid_n"], alpha=2e-3))
        else:
            work += r["n"] * 40.0
    scale = work / capacity / (load * reqs[-1]["arrival"])
    loop = serving.ServingLoop(8 << 30, max_instances=4096)
    clocks = ClockSampler(0)
    clocks.start()
    try:
        o = loop.serve(reqs, time_scale=scale)
    finally:
        loop.close()
    clk = clocks.stop()
    pl = serving.serve_plain(reqs, time_scale=scale)
    return {
        "metric": "served solves/s and p50/p99 latency", "offered_load": load,
        "value": o["solves_per_s"], "unit": "solves/s",
        "latency_s": {"p50": o["p50"], "p99": o["p99"], "max": float(np.max(o["latency"]))},
        "plain_form": {"value": pl["solves_per_s"], "unit": "solves/s", "p50": pl["p50"], "p99": pl["p99"],
                       "sample": "the same requests and arrivals, one at a time, first come first served"},
        "config": {"workload": f"served: first {len(reqs)} of the 20,000 seeded requests (seed 7), "
                               f"{100.0 * len(reqs) / 20000:.1f} % of the stream",
                   "arrival_time_scale": scale, "arena_gb": 8,
                   "launches": "time slices of about 4 ms (sweeps per launch from the measured sweep time)"},
        "admission_refusals": o["refusals"], "makespan_s": o["makespan"], "clocks": clk,
    }


MIXED_CHECK_TE = 0.004


def mixed_error_vs_fp64(rk, prob, y0, method):
    """The mixed form's error, stated with its result: relative max-norm difference at
    t = MIXED_CHECK_TE between the mixed form and the exact FP64 form (which is
    bit-identical to the reference) from the same initial values at tol 1e-6.  A short
    interval keeps the FP64 solve to a few seconds at N=4000; the full-interval errors
    at N up to 2000 are in the mixed-precision tests."""
    with rk.Solver(prob, method=method, precision="exact") as s:
        ref, rst = s.solve(T0, MIXED_CHECK_TE, y0, TOL)
    with rk.Solver(prob, method=method, precision="mixed") as s:
        y, st = s.solve(T0, MIXED_CHECK_TE, y0, TOL)
    err = float(np.max(np.abs(y - ref)) / np.max(np.abs(ref)))
    return {"t_end": MIXED_CHECK_TE, "rel_max_norm": err, "tol": TOL, "within_tol": err <= TOL,
            "steps_mixed": st["steps_acc"] + st["steps_rej"], "steps_fp64": rst["steps_acc"] + rst["steps_rej"]}


def run_batched(args):
    """Batched form: a seeded sample of the 4096-instance BRUSS2D-MIX distribution
    (N log-uniform [16,512], alpha U[1e-3,1e-2], tol log-uniform [1e-8,1e-4],
    DOPRI5(4), t in [0, 0.5]) in one batch; solves/s with y0 already in HBM, and
    the same instances' work through the plain form and the CPU port for comparison."""
    import concurrent.futures as cf

    import torch

    import rk_gb300 as rk
    from rk_gb300 import workloads

    insts = workloads.batched_instances(4096, seed=2024)
    rng = np.random.default_rng(5)
    sample = [insts[i] for i in sorted(rng.choice(len(insts), args.instances, replace=False))]
    probs = [rk.bruss2d_mix(d["grid_n"], d["alpha"]) for d in sample]
    y0s = [rk.ode_start(p) for p in probs]
    arena = sum(rk.footprint(p, 7) for p in probs) + (64 << 20)
    torch.cuda.init()
    with rk.Batch(arena, len(sample) + 1, precision=args.precision) as b:
        t_e2e = time.perf_counter()
        for k, (p, y0, d) in enumerate(zip(probs, y0s, sample)):
            assert b.add(p, y0, d["t0"], d["te"], d["tol"], host_id=k) is not None
        torch.cuda.synchronize()
        tuned_ns = b.tune(2)
        stream = torch.cuda.ExternalStream(b.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks = ClockSampler(0)
        clocks.start()
        ev0.record(stream)
        sweeps = 0
        while b.run(args.sweeps_per_launch) > 0:
            sweeps += args.sweeps_per_launch
        ev1.record(stream)
        ev1.synchronize()
        clk = clocks.stop()
        ms = ev0.elapsed_time(ev1)
        results = {}
        for slot in b.finished():
            y, st, hid = b.take(slot)
            results[hid] = (y, st)
        e2e_s = time.perf_counter() - t_e2e
        info = b.info()
        tuning = b.tuning()
    comp_steps = sum(2 * d["grid_n"] ** 2 * (results[k][1]["steps_acc"] + results[k][1]["steps_rej"])
                     for k, d in enumerate(sample))
    value = len(sample) / (ms * 1e-3)

    # plain form, one solve after another: on every instance (--plain-sample 0), or on
    # a sub-sample with its time scaled by component-steps
    if args.plain_sample <= 0:
        sub = list(range(len(sample)))
    else:
        sub = list(range(0, len(sample), max(1, len(sample) // args.plain_sample)))[: args.plain_sample]
    t = time.perf_counter()
    same = 0
    for k in sub:
        with rk.Solver(probs[k], method="DOPRI54", precision=args.precision) as s:
            y, st = s.solve(0.0, 0.5, y0s[k], sample[k]["tol"])
        same += int(np.array_equal(y, results[k][0]))
    plain_s = time.perf_counter() - t
    sub_cs = sum(2 * sample[k]["grid_n"] ** 2 * (results[k][1]["steps_acc"] + results[k][1]["steps_rej"])
                 for k in sub)
    plain_value = len(sample) / (plain_s * comp_steps / max(1, sub_cs))
    plain_note = ("every instance, one solve after another" if len(sub) == len(sample) else
                  f"{len(sub)} instances solved one after another, scaled by work")

    line = {
        "metric": "batched BRUSS2D-MIX solves/s (4096-instance distribution)", "value": value,
        "unit": "solves/s", "n_gpus": 1, "steps": sweeps, "warmup": 0,
        "ms_per_step": ms / max(1, sweeps), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded instance list)",
        "config": {"workload": f"batched: {len(sample)} of 4096 seeded instances (seed 2024)",
                   "precision": args.precision, "tuning": tuning,
                   "tuned_ns_per_pair_step": tuned_ns,
                   "component_steps": comp_steps},
        "component_steps_per_s": comp_steps / (ms * 1e-3),
        "plain_form": {"value": plain_value, "unit": "solves/s", "sample": plain_note,
                       "results_bit_identical_to_batch": same},
        "host_pow_steps": sum(results[k][1]["host_pow_steps"] for k in results),
        "e2e": {"value": len(sample) / e2e_s, "unit": "solves/s",
                "h2d_bytes_per_step": sum(8 * p.n for p in probs) / max(1, sweeps),
                "d2h_bytes_per_step": sum(8 * p.n for p in probs) / max(1, sweeps)},
        "gpu_launches": info["launches"], "clocks": clk,
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import rk_oracle
        rk_oracle.load()
        threads = os.cpu_count() or 1
        order = sorted(range(len(sample)), key=lambda k: workloads.estimated_work(sample[k]))
        picked, budget = [], 15.0 * threads * 3e7  # about 15 s at ~3e7 component-steps/s per core
        acc = 0.0
        for k in order:
            if acc + workloads.estimated_work(sample[k]) > budget:
                continue
            picked.append(k)
            acc += workloads.estimated_work(sample[k])
        def one(k):
            d = sample[k]
            return port_solve(rk_oracle, y0s[k], d["tol"], 0, 1, grid_n=d["grid_n"],
                              alpha=d["alpha"], t0=0.0, te=0.5)
        t = time.perf_counter()
        with cf.ThreadPoolExecutor(threads) as ex:
            outs = list(ex.map(one, picked))
        cpu_s = time.perf_counter() - t
        cpu_cs = sum(2 * sample[k]["grid_n"] ** 2 * (o[1]["steps_acc"] + o[1]["steps_rej"])
                     for k, o in zip(picked, outs))
        line["cpu_baseline"] = {"value": len(sample) / (cpu_s * comp_steps / max(1, cpu_cs)),
                                "unit": "solves/s", "cores": threads, "kind": "port",
                                "sample": f"{len(picked)} of the instances, one per thread "
                                          f"({cpu_s:.1f} s), scaled by work"}
    print(json.dumps(line), flush=True)
    return 0


def run_served(args):
    """Serving: a prefix of the seeded 20,000-request Poisson stream (half BRUSS2D-MIX
    N log-uniform [32,1024] t in [0,0.5], half banded LV n log-uniform [1e3,1e6]
    t in [0,10], tol 1e-6), arrivals rescaled so the offered load is --load times
    the GPU's measured batched throughput; continuous batching with admission by
    HBM footprint into an arena of --arena-gb.  Reports solves/s and p50/p99
    latency, and the plain form serving the same stream one request at a time."""
    import rk_gb300 as rk
    from rk_gb300 import serving, workloads

    reqs = workloads.served_requests(20000, seed=7)[: args.requests]
    # capacity estimate: component-steps of the sample at the batched rate measured
    # on this part (5.3e9 component-steps/s in the FP64 exact mode, 1024 instances)
    work = 0.0
    for r in reqs:
        if r["kind"] == "bruss":
            work += workloads.estimated_work(dict(grid_n=r["grid_n"], alpha=2e-3))
        else:
            work += r["n"] * 40.0
    busy = work / 5.3e9
    span = reqs[-1]["arrival"]
    scale = busy / (args.load * span)
    loop = serving.ServingLoop(int(args.arena_gb * (1 << 30)), max_instances=4096,
                               sweeps_per_launch=args.sweeps_per_launch, precision=args.precision)
    clocks = ClockSampler(0)
    clocks.start()
    try:
        out = loop.serve(reqs, time_scale=scale)
    finally:
        loop.close()
    clk = clocks.stop()
    line = {
        "metric": "served solves/s and p50/p99 latency (BRUSS2D-MIX + banded LV stream)",
        "value": out["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": len(reqs),
        "warmup": 0, "ms_per_step": 1e3 * out["makespan"] / len(reqs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Poisson request stream)",
        "config": {"workload": f"served: first {len(reqs)} of 20,000 seeded requests (seed 7)",
                   "offered_load": args.load, "arrival_time_scale": scale,
                   "arena_gb": args.arena_gb, "sweeps_per_launch": args.sweeps_per_launch,
                   "precision": args.precision},
        "latency_s": {"p50": out["p50"], "p99": out["p99"], "max": float(np.max(out["latency"]))},
        "admission_refusals": out["refusals"], "makespan_s": out["makespan"], "clocks": clk,
    }
    if args.plain_requests != 0:
        sub = reqs if args.plain_requests < 0 else reqs[: args.plain_requests]
        pl = serving.serve_plain(sub, time_scale=scale, precision=args.precision)
        line["plain_form"] = {"value": pl["solves_per_s"], "unit": "solves/s",
                              "p50": pl["p50"], "p99": pl["p99"],
                              "sample": f"first {len(sub)} requests, one at a time, same arrivals"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "served"])
    ap.add_argument("--variant", default="d", choices=["d", "lowstorage"],
                    help="d: stage vectors in HBM (default); lowstorage: wavefront with ring buffers")
    ap.add_argument("--block-rows", type=int, default=0)
    ap.add_argument("--flow-skew", type=int, default=0,
                    help="plain form, schedule 3: wavefront skew in tiles (0 = automatic)")
    ap.add_argument("--schedule", type=int, default=0,
                    help="plain form stage synchronisation: 0 auto, 1 grid barrier, 2 neighbour flags")
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--load", type=float, default=0.5)
    ap.add_argument("--arena-gb", type=float, default=8.0)
    ap.add_argument("--plain-requests", type=int, default=-1,
                    help="served: requests the plain form serves for comparison (-1: all)")
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--sweeps-per-launch", type=int, default=256)
    ap.add_argument("--plain-sample", type=int, default=32)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="DOPRI54")
    ap.add_argument("--grid", type=int, default=GRID_N,
                    help="grid size N (2000 is the benchmark; smaller only for profiling)")
    ap.add_argument("--precision", default="exact", choices=["exact", "exact-hwmul", "fma", "mixed"],
                    help="exact (default): bit-identical to the reference; fma: fewer FP64 "
                         "instructions; mixed: FP32 stage vectors (the N=4000 configuration)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched, served and mixed-precision records of the default run")
    ap.add_argument("--batched-sample", type=int, default=128,
                    help="instances of the 4096-instance list in the default run's batched record")
    ap.add_argument("--served-requests", type=int, default=200,
                    help="requests of the 20,000-request stream per load in the served record")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        if args.sweeps_per_launch == 256:
            args.sweeps_per_launch = 0  # time slices
        return run_served(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

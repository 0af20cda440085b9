#!/usr/bin/env python3
"""Generate golden fixtures by running the reference solver itself.

Each case is compiled from the reference sources (oracle/Makefile, `ref`
target: the reference's tools.c, methods.c, threads.c, one problem module and
one solver variant, plus oracle/ref_harness.c as main) with the case's
compile-time DEFINES, run, and recorded as JSON under tests/golden/:

  steps / accepted / rejected  -- from "Number of steps: ..." (src/tools.c:69)
  y_sha256, y_first/last/min/max -- final state, bit for bit (float.hex)
  y_hex                        -- the whole final state for small systems
  y_sample                     -- every k-th component for large systems
  h_trace, t_trace             -- h and t of every attempted step, from the
                                  reference's -DDUMP trajectory (tools.h:239-256)
  dump_sha256, dump_bytes      -- the DUMP file itself (t, h and the candidate
                                  state of every step as %.20e), for small systems

Run here, where the reference sources exist:
    python tests/golden/make_golden.py [--only NAME ...] [--big]
The fixtures are committed; the tests never read the reference at run time.
"""
import argparse
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("RK_REFERENCE", "/root/reference")

# name, problem, variant, defines, dump-trace?, threads
CASES = [
    # BRUSS2D-MIX, the headline CPU configuration (N=250) and DOPRI87 beside it
    ("bruss_n250_dopri54_tol1e-6", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=250, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n250_dopri87_tol1e-6", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=250, BRUSS_ALPHA="2e-3", METHOD="DOPRI87", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    # small grids: every boundary branch of bruss2d-mix.c:66-206
    ("bruss_n2_dopri54", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=2, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n3_dopri54", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=3, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n4_dopri54", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=4, BRUSS_ALPHA="1e-2", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n5_dopri87", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=5, BRUSS_ALPHA="2e-3", METHOD="DOPRI87", TOL="1e-8", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n8_dopri54", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=8, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n16_a1e-2_tol1e-8", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=16, BRUSS_ALPHA="1e-2", METHOD="DOPRI54", TOL="1e-8", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n16_a1e-3_tol1e-4", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=16, BRUSS_ALPHA="1e-3", METHOD="DOPRI54", TOL="1e-4", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n64_dopri87_tol1e-7", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=64, BRUSS_ALPHA="5e-3", METHOD="DOPRI87", TOL="1e-7", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n100_dopri54_tol1e-6", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=100, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), True, 1),
    # the other tableaux of methods.c (embedded and fixed-step)
    ("bruss_n32_rkf23", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="RKF23", TOL="1e-5", T_END="0.2", STEP_LIMIT=0), True, 1),
    ("bruss_n32_verner65", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="VERNER65", TOL="1e-7", T_END="0.5", STEP_LIMIT=0), True, 1),
    ("bruss_n32_heun2_fixed", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="HEUN2", T_END="0.5", STEP_LIMIT=200), True, 1),
    ("bruss_n32_rk4_fixed", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="RK4", T_END="0.5", STEP_LIMIT=100), True, 1),
    ("bruss_n32_ssprk3_fixed", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="SSPRK3", T_END="0.5", STEP_LIMIT=150), True, 1),
    # STEP_LIMIT truncation (config.h:71 default behaviour)
    ("bruss_n32_steplimit20", "bruss2d-mix", "seq/D",
     dict(BRUSS_GRID_SIZE=32, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-9", T_END="0.1", STEP_LIMIT=20), True, 1),
    # the reference's LV pairs module (lv.c)
    ("lv_pairs_1000_dopri54", "lv", "seq/D",
     dict(LV_COUNT=1000, METHOD="DOPRI54", TOL="1e-6", T_END="10.0", STEP_LIMIT=0), True, 1),
    ("lv_pairs_10000_dopri87", "lv", "seq/D",
     dict(LV_COUNT=10000, METHOD="DOPRI87", TOL="1e-9", T_END="10.0", STEP_LIMIT=0), False, 1),
    # larger grids (pthreads D: bit-identical to seq D, faster to generate)
    ("bruss_n512_a1e-3_tol1e-4", "bruss2d-mix", "pthreads/D",
     dict(BRUSS_GRID_SIZE=512, BRUSS_ALPHA="1e-3", METHOD="DOPRI54", TOL="1e-4", T_END="0.5", STEP_LIMIT=0), False, 8),
]

BIG_CASES = [
    ("bruss_n512_a1e-2_tol1e-8", "bruss2d-mix", "pthreads/PipeD4ls",
     dict(BRUSS_GRID_SIZE=512, BRUSS_ALPHA="1e-2", METHOD="DOPRI54", TOL="1e-8", T_END="0.5", STEP_LIMIT=0), False, 8),
    # the N=2000 FP64 configuration, both tableaux (minutes of CPU time each)
    ("bruss_n2000_dopri54_tol1e-6", "bruss2d-mix", "pthreads/PipeD4ls",
     dict(BRUSS_GRID_SIZE=2000, BRUSS_ALPHA="2e-3", METHOD="DOPRI54", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), False, 8),
    ("bruss_n2000_dopri87_tol1e-6", "bruss2d-mix", "pthreads/PipeD4ls",
     dict(BRUSS_GRID_SIZE=2000, BRUSS_ALPHA="2e-3", METHOD="DOPRI87", TOL="1e-6", T_END="0.5", STEP_LIMIT=0), False, 8),
]

FULL_Y_MAX = 4096       # store every component up to this size
SAMPLE_TARGET = 2048    # otherwise about this many evenly spaced components


def hx(v):
    return float(v).hex()


def build(name, problem, variant, defines, dump):
    d = dict(defines)
    if dump:
        d["DUMP"] = 1
    dstr = " ".join(f"{k}={v}" for k, v in d.items())
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", f"NAME=g_{name}",
                    f"VARIANT={variant}", f"PROBLEM={problem}", f"DEFINES={dstr}", f"REF={REF}"],
                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return os.path.join(REPO, "oracle", "_ref", f"g_{name}")


def run_case(case):
    name, problem, variant, defines, dump, threads = case
    exe = build(name, problem, variant, defines, dump)
    with tempfile.TemporaryDirectory() as td:
        ybin = os.path.join(td, "y.bin")
        env = dict(os.environ, RK_DUMP_Y=ybin, NUM_THREADS=str(threads))
        out = subprocess.run([exe], cwd=td, env=env, check=True, capture_output=True, text=True).stdout
        y = np.fromfile(ybin, dtype="<f8")
        trace = None
        if dump:
            trace, ttrace = [], []
            dpath = os.path.join(td, "DUMP")
            with open(dpath) as f:
                for line in f:
                    t_s, h_s = line.split("\t", 2)[:2]
                    trace.append(float(h_s))
                    ttrace.append(float(t_s))
            with open(dpath, "rb") as f:
                dump_raw = f.read()
    m = re.search(r"Number of steps: (\d+) \((\d+) accepted, (\d+) rejected\)", out)
    steps, acc, rej = map(int, m.groups())
    n = y.size
    rec = {
        "name": name,
        "problem": {"bruss2d-mix": "bruss2d-mix", "lv": "lv-pairs"}[problem],
        "reference_variant": variant,
        "defines": {k: str(v) for k, v in defines.items()},
        "n": int(n),
        "method": defines.get("METHOD", "DOPRI54"),
        "tol": float(defines.get("TOL", 0.0)) if defines.get("METHOD") not in ("HEUN2", "RK4", "SSPRK3") else 0.0,
        "t0": 0.0,
        "t_end": float(defines["T_END"]),
        "step_limit": int(defines["STEP_LIMIT"]),
        "steps": steps, "accepted": acc, "rejected": rej,
        "step_limit_reached": "Step limit reached" in out,
        "y_sha256": hashlib.sha256(y.astype("<f8").tobytes()).hexdigest(),
        "y_first": hx(y[0]), "y_last": hx(y[-1]), "y_min": hx(y.min()), "y_max": hx(y.max()),
        "result_line": [l for l in out.splitlines() if l.startswith("Result:")][0],
    }
    if problem == "bruss2d-mix":
        rec["grid_n"] = int(defines["BRUSS_GRID_SIZE"])
        rec["alpha"] = float(defines["BRUSS_ALPHA"])
    if n <= FULL_Y_MAX:
        rec["y_hex"] = [hx(v) for v in y]
    else:
        stride = max(1, n // SAMPLE_TARGET) | 1
        rec["y_sample"] = {"stride": stride, "values": [hx(v) for v in y[::stride]]}
    if trace is not None:
        # the trace holds the h of every attempted step; a DUMP line is written
        # per step_control call (tools.h:239-256)
        rec["h_trace"] = [hx(v) for v in trace]
        rec["t_trace"] = [hx(v) for v in ttrace]
        if n <= FULL_Y_MAX:
            rec["dump_sha256"] = hashlib.sha256(dump_raw).hexdigest()
            rec["dump_bytes"] = len(dump_raw)
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--big", action="store_true", help="also the N=512/N=2000 cases (minutes each)")
    args = ap.parse_args()
    if not os.path.isdir(os.path.join(REF, "src")):
        sys.exit(f"reference sources not found at {REF}")
    cases = CASES + (BIG_CASES if args.big else [])
    if args.only:
        cases = [c for c in cases if c[0] in args.only]
    for c in cases:
        rec = run_case(c)
        path = os.path.join(HERE, f"{rec['name']}.json")
        with open(path, "w") as f:
            json.dump(rec, f, indent=0)
        print(f"{rec['name']}: {rec['steps']} ({rec['accepted']}/{rec['rejected']}) n={rec['n']}", flush=True)


if __name__ == "__main__":
    main()

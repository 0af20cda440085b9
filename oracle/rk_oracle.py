"""ctypes wrapper of the CPU oracle (oracle/rk_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Loaded by the tests, the smoke check and the benchmark's CPU-baseline leg; the
GPU product never imports it.  See rk_oracle.h for what the oracle restates
(the reference's seq/D.c step loop, tools.h step control, methods.c tableaux,
bruss2d-mix.c and lv.c) and how it is pinned to the reference.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "librk_oracle.so")

BRUSS2D_MIX, LV_PAIRS, LV_BANDED = 0, 1, 2
MAXS = 16


class Tableau(ctypes.Structure):
    _fields_ = [("s", ctypes.c_int), ("ord", ctypes.c_int), ("embedded", ctypes.c_int),
                ("A", ctypes.c_double * (MAXS * MAXS)), ("b", ctypes.c_double * MAXS),
                ("b_hat", ctypes.c_double * MAXS), ("c", ctypes.c_double * MAXS)]


class Problem(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n", ctypes.c_int), ("grid_n", ctypes.c_int),
                ("alpha", ctypes.c_double), ("lv_r", ctypes.c_void_p), ("lv_a", ctypes.c_void_p)]


class Stats(ctypes.Structure):
    _fields_ = [("steps_acc", ctypes.c_int), ("steps_rej", ctypes.c_int),
                ("t", ctypes.c_double), ("h", ctypes.c_double)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        _lib.ork_solve.restype = ctypes.c_int
        _lib.ork_eval_comp.restype = ctypes.c_double
        _lib.ork_h_new.restype = ctypes.c_double
        _lib.ork_h_new.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    return _lib


def tableau(name):
    t = Tableau()
    if load().ork_tableau_get(name.encode(), ctypes.byref(t)) != 0:
        raise KeyError(name)
    s = t.s
    A = np.frombuffer(t.A, dtype=np.float64).reshape(MAXS, MAXS)[:s, :s].copy()
    return dict(s=s, ord=t.ord, embedded=bool(t.embedded), A=A,
                b=np.array(t.b[:s]), b_hat=np.array(t.b_hat[:s]), c=np.array(t.c[:s]))


def _problem(kind, n, grid_n=0, alpha=0.0, lv_r=None, lv_a=None):
    keep = []
    r = a = None
    if lv_r is not None:
        lr = np.ascontiguousarray(lv_r, dtype=np.float64)
        la = np.ascontiguousarray(lv_a, dtype=np.float64)
        keep += [lr, la]
        r, a = lr.ctypes.data, la.ctypes.data
    return Problem(kind, n, grid_n, alpha, r, a), keep


def h_new(h, err, tol, ord):
    return load().ork_h_new(h, err, tol, ord)


def bruss_start(N):
    y0 = np.zeros(2 * N * N)
    load().ork_bruss_start(N, y0.ctypes.data_as(ctypes.c_void_p))
    return y0


def lv_pairs_start(n):
    y0 = np.zeros(n)
    load().ork_lv_pairs_start(n, y0.ctypes.data_as(ctypes.c_void_p))
    return y0


def eval_all(kind, y, grid_n=0, alpha=0.0, lv_r=None, lv_a=None):
    y = np.ascontiguousarray(y, dtype=np.float64)
    p, keep = _problem(kind, y.size, grid_n, alpha, lv_r, lv_a)
    f = np.zeros_like(y)
    load().ork_eval_all(ctypes.byref(p), y.ctypes.data_as(ctypes.c_void_p),
                        f.ctypes.data_as(ctypes.c_void_p))
    return f


def solve(kind, y0, method, t0, te, tol, step_limit=0, grid_n=0, alpha=0.0, lv_r=None,
          lv_a=None, threads=1, trace=False, rows=0):
    """Returns (y, dict(steps_acc, steps_rej, t, h, h_trace)).  rows > 0 selects the
    pipelined schedule (BRUSS2D-MIX) with blocks of that many grid rows."""
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p, keep = _problem(kind, y0.size, grid_n, alpha, lv_r, lv_a)
    t = Tableau()
    if load().ork_tableau_get(method.encode(), ctypes.byref(t)) != 0:
        raise KeyError(method)
    y = np.empty_like(y0)
    st = Stats()
    cap = 1 << 20 if trace else 0
    tr = np.zeros(cap) if trace else None
    rc = _lib.ork_solve_pipelined(ctypes.byref(p), ctypes.byref(t), ctypes.c_double(t0),
                                  ctypes.c_double(te), y0.ctypes.data_as(ctypes.c_void_p),
                                  y.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(tol),
                                  int(step_limit), ctypes.byref(st),
                                  tr.ctypes.data_as(ctypes.c_void_p) if trace else None, cap,
                                  int(threads), int(rows))
    if rc != 0:
        raise RuntimeError(f"ork_solve failed: {rc}")
    out = dict(steps_acc=st.steps_acc, steps_rej=st.steps_rej, t=st.t, h=st.h)
    if trace:
        out["h_trace"] = tr[:st.steps_acc + st.steps_rej].copy()
    return y, out

"""GB300 embedded Runge-Kutta step loop: Python host mirror of the reference's C interface.

The reference exposes `void solver(double t0, double te, double *y0, double *y,
double tol)` (include/solver.h:47) with the problem chosen at link time
(include/ode.h) and the tableau by the METHOD macro (include/config.h:88-90,
src/methods.c).  This module mirrors that contract over the C ABI of
librkcu.so (include/rkcu.h) through ctypes:

    y, stats = solver(0.0, 0.5, y0, None, 1e-6, problem=bruss2d_mix(250, 2e-3))

The GPU library is required: importing works anywhere, but every compute call
raises RkcuError when librkcu.so is missing or no GPU is present -- there is
no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librkcu.so")

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_TIMEOUT = -4
ERR_STATE = -5
ERR_NO_DEVICE = -6
ERR_TOO_LARGE = -7
ERR_RHS = -8

PROBLEM_BRUSS2D_MIX = 0
PROBLEM_LV_PAIRS = 1
PROBLEM_LV_BANDED = 2
PROBLEM_RHS = 3

FP64_EXACT = 0
FP64_FMA = 1
MIXED = 2
FP64_EXACT_HWMUL = 3

VARIANT_D = 0
VARIANT_LOWSTORAGE = 1

METHODS = ("HEUN2", "RK4", "SSPRK3", "RKF23", "DOPRI54", "VERNER65", "DOPRI87")
EMBEDDED = {"HEUN2": False, "RK4": False, "SSPRK3": False, "RKF23": True,
            "DOPRI54": True, "VERNER65": True, "DOPRI87": True}

# Symbols include/rkcu.h declares; tests check the library exports each one.
EXPORTS = (
    "rkcu_options_default", "rkcu_create", "rkcu_destroy", "rkcu_set_method",
    "rkcu_set_method_by_name", "rkcu_builtin_method", "rkcu_solve", "rkcu_begin",
    "rkcu_advance", "rkcu_query", "rkcu_get_y", "rkcu_stream", "rkcu_launch_count",
    "rkcu_device_bytes", "rkcu_ode_start", "rkcu_ode_eval_rng", "rkcu_ode_acc_dist",
    "rkcu_strerror", "rkcu_last_cuda_error", "rkcu_debug_inject_wait_timeout",
    "rkcu_step_size", "rkcu_step_sizes_device", "rkcu_run", "rkcu_solve_noalloc",
    "rkcu_batch_footprint", "rkcu_batch_create", "rkcu_batch_destroy", "rkcu_batch_add",
    "rkcu_batch_run", "rkcu_batch_finished", "rkcu_batch_take", "rkcu_batch_tune",
    "rkcu_batch_set_tuning", "rkcu_batch_get_tuning", "rkcu_batch_info", "rkcu_batch_stream",
    "rkcu_set_trace", "rkcu_get_trace", "rkcu_set_rhs", "rkcu_rhs_builtin",
)

# int rhs(double t, const double *w, double *f, int n, void *stream, void *user)
RHS_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p)


class RkcuError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = f"{what}: status {status}"
        if _lib is not None:
            msg += f" ({_lib.rkcu_strerror(status).decode()})"
            extra = _lib.rkcu_last_cuda_error().decode()
            if extra:
                msg += f" [{extra}]"
        super().__init__(msg)


class Problem(ctypes.Structure):
    _fields_ = [("problem", ctypes.c_int), ("n", ctypes.c_int), ("grid_n", ctypes.c_int),
                ("alpha", ctypes.c_double), ("lv_r", ctypes.c_void_p), ("lv_a", ctypes.c_void_p)]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("variant", ctypes.c_int),
                ("step_limit", ctypes.c_int), ("device", ctypes.c_int),
                ("stream", ctypes.c_void_p), ("wait_timeout_s", ctypes.c_double),
                ("h_init", ctypes.c_double), ("block_rows", ctypes.c_int),
                ("schedule", ctypes.c_int), ("flow_skew", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("steps_acc", ctypes.c_int), ("steps_rej", ctypes.c_int), ("t", ctypes.c_double),
                ("h", ctypes.c_double), ("done", ctypes.c_int), ("step_limit_reached", ctypes.c_int),
                ("host_pow_steps", ctypes.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load():
    """Load librkcu.so (built by rk_gb300.build); raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RkcuError(ERR_NO_DEVICE, f"{LIB_PATH} is not built (run rk_gb300.build)")
    lib = ctypes.CDLL(LIB_PATH)
    P, D, I, V = ctypes.POINTER, ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    lib.rkcu_strerror.restype = ctypes.c_char_p
    lib.rkcu_strerror.argtypes = [I]
    lib.rkcu_last_cuda_error.restype = ctypes.c_char_p
    lib.rkcu_options_default.argtypes = [P(Options)]
    lib.rkcu_create.argtypes = [P(V), P(Problem), P(Options)]
    lib.rkcu_destroy.argtypes = [V]
    lib.rkcu_set_method.argtypes = [V, P(P(D)), V, V, V, I, I]
    lib.rkcu_set_method_by_name.argtypes = [V, ctypes.c_char_p]
    lib.rkcu_builtin_method.argtypes = [ctypes.c_char_p, V, V, V, V, P(I), P(I), P(I)]
    lib.rkcu_solve.argtypes = [V, D, D, V, V, D, P(Stats)]
    lib.rkcu_begin.argtypes = [V, D, D, V, I, D]
    lib.rkcu_advance.argtypes = [V, I]
    lib.rkcu_query.argtypes = [V, P(Stats)]
    lib.rkcu_get_y.argtypes = [V, V, I]
    lib.rkcu_stream.restype = V
    lib.rkcu_stream.argtypes = [V]
    lib.rkcu_launch_count.restype = ctypes.c_longlong
    lib.rkcu_launch_count.argtypes = [V]
    lib.rkcu_device_bytes.restype = ctypes.c_longlong
    lib.rkcu_device_bytes.argtypes = [V]
    lib.rkcu_ode_start.argtypes = [P(Problem), D, V]
    lib.rkcu_ode_eval_rng.argtypes = [P(Problem), I, I, D, V, V]
    lib.rkcu_ode_acc_dist.argtypes = [P(Problem)]
    lib.rkcu_debug_inject_wait_timeout.argtypes = [V, I]
    lib.rkcu_step_size.restype = D
    lib.rkcu_step_size.argtypes = [D, D, D, I, P(I)]
    lib.rkcu_step_sizes_device.argtypes = [V, V, I, D, I, V, V]
    lib.rkcu_run.argtypes = [V, I, P(Stats)]
    lib.rkcu_set_rhs.argtypes = [V, V, V]
    lib.rkcu_set_trace.argtypes = [V, I, I]
    lib.rkcu_get_trace.argtypes = [V, V, V, V, V, I, P(I)]
    LL = ctypes.c_longlong
    lib.rkcu_batch_footprint.restype = LL
    lib.rkcu_batch_footprint.argtypes = [P(Problem), I]
    lib.rkcu_batch_create.argtypes = [P(V), LL, I, ctypes.c_char_p, P(Options)]
    lib.rkcu_batch_destroy.argtypes = [V]
    lib.rkcu_batch_add.argtypes = [V, P(Problem), D, D, D, V, LL, P(I)]
    lib.rkcu_batch_run.argtypes = [V, I, P(I)]
    lib.rkcu_batch_finished.argtypes = [V, V, I, P(I)]
    lib.rkcu_batch_take.argtypes = [V, I, V, P(Stats), P(LL)]
    lib.rkcu_batch_tune.argtypes = [V, I, P(D)]
    lib.rkcu_batch_set_tuning.argtypes = [V, I, I, I, I]
    lib.rkcu_batch_get_tuning.argtypes = [V, P(I), P(I), P(I)]
    lib.rkcu_batch_info.argtypes = [V, P(I), P(LL), P(LL)]
    lib.rkcu_batch_stream.restype = V
    lib.rkcu_batch_stream.argtypes = [V]
    lib.rkcu_solve_noalloc.argtypes = [P(Problem), ctypes.c_char_p, I, I, D, D, V, V, D, V, P(Stats)]
    _lib = lib
    return lib


def _check(rc, what):
    if rc != OK:
        raise RkcuError(rc, what)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


# --------------------------------------------------------------------------
# Problem constructors (the ode.h modules, with run-time parameters)
# --------------------------------------------------------------------------
class ProblemSpec:
    """A problem instance; keeps any parameter arrays alive for the C side."""

    def __init__(self, kind, n, grid_n=0, alpha=0.0, lv_r=None, lv_a=None):
        self.kind, self.n, self.grid_n, self.alpha = kind, int(n), int(grid_n), float(alpha)
        self.lv_r = None if lv_r is None else np.ascontiguousarray(lv_r, dtype=np.float64)
        self.lv_a = None if lv_a is None else np.ascontiguousarray(lv_a, dtype=np.float64)

    def cstruct(self):
        return Problem(self.kind, self.n, self.grid_n, self.alpha,
                       None if self.lv_r is None else self.lv_r.ctypes.data,
                       None if self.lv_a is None else self.lv_a.ctypes.data)

    @property
    def name(self):
        return {PROBLEM_BRUSS2D_MIX: "bruss2d-mix", PROBLEM_LV_PAIRS: "lv-pairs",
                PROBLEM_LV_BANDED: "lv-banded", PROBLEM_RHS: "rhs"}[self.kind]


def rhs_problem(n):
    """A system of n components whose right-hand side the caller supplies
    (Solver.set_rhs): any ode_eval_rng, without a limited access distance."""
    return ProblemSpec(PROBLEM_RHS, n)


class DeviceArray:
    """A device array of n doubles at a raw address, for torch.as_tensor (the
    CUDA array interface); lets a Python right-hand side work on w and f."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 3, "strides": None}


def bruss2d_mix(grid_n, alpha=2e-3):
    """BRUSS2D-MIX (src/problems/bruss2d-mix.c) on an N x N grid, n = 2 N^2."""
    return ProblemSpec(PROBLEM_BRUSS2D_MIX, 2 * grid_n * grid_n, grid_n, alpha)


def lv_pairs(count):
    """The reference's LV module (src/problems/lv.c) with LV_COUNT pairs."""
    return ProblemSpec(PROBLEM_LV_PAIRS, 2 * count)


def lv_banded(r, a):
    """Banded LV chain dy_i = y_i (r_i + sum_{|j-i|<=2} a_ij y_j); a has shape (n, 5)."""
    r = np.asarray(r, dtype=np.float64)
    a = np.asarray(a, dtype=np.float64).reshape(r.size, 5)
    return ProblemSpec(PROBLEM_LV_BANDED, r.size, lv_r=r, lv_a=a)


def lv_banded_random(n, seed):
    """Seeded banded LV instance: r ~ U[0.5,1.5], a_ii = -1, a_ij ~ U[-0.1,0.1] for
    0 < |i-j| <= 2 (truncated at the ends), y0 ~ U[0.5,1.5].  Returns (problem, y0)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.5, 1.5, n)
    a = rng.uniform(-0.1, 0.1, (n, 5))
    a[:, 2] = -1.0
    a[0, 0] = a[0, 1] = a[1, 0] = 0.0
    a[n - 1, 4] = a[n - 1, 3] = a[n - 2, 4] = 0.0
    y0 = rng.uniform(0.5, 1.5, n)
    return lv_banded(r, a), y0


def builtin_method(name):
    """Tableau of src/methods.c by name: dict(A (s,s), b, b_hat, c, s, ord, embedded)."""
    lib = load()
    A = np.zeros(256)
    b, bh, c = np.zeros(16), np.zeros(16), np.zeros(16)
    s, o, e = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib.rkcu_builtin_method(name.encode(), _ptr(A), _ptr(b), _ptr(bh), _ptr(c),
                                   ctypes.byref(s), ctypes.byref(o), ctypes.byref(e)),
           f"builtin_method({name})")
    S = s.value
    return dict(A=A[:S * S].reshape(S, S).copy(), b=b[:S].copy(), b_hat=bh[:S].copy(),
                c=c[:S].copy(), s=S, ord=o.value, embedded=bool(e.value))


def ode_start(problem, t=0.0):
    """ode_start (include/ode.h:32) for BRUSS2D-MIX and LV pairs."""
    lib = load()
    y0 = np.zeros(problem.n)
    ps = problem.cstruct()
    _check(lib.rkcu_ode_start(ctypes.byref(ps), t, _ptr(y0)), "ode_start")
    return y0


def ode_eval_rng(problem, i, j, t, y):
    """ode_eval_rng (include/ode.h:34) evaluated by the device evaluator: returns f
    with f[i..j] filled (global indexing), other entries zero."""
    lib = load()
    y = np.ascontiguousarray(y, dtype=np.float64)
    f = np.zeros(problem.n)
    ps = problem.cstruct()
    _check(lib.rkcu_ode_eval_rng(ctypes.byref(ps), i, j, t, _ptr(y), _ptr(f)), "ode_eval_rng")
    return f


def ode_acc_dist(problem):
    ps = problem.cstruct()
    return load().rkcu_ode_acc_dist(ctypes.byref(ps))


def step_sizes(h, err, tol, ord, device=False):
    """Step-size updates h * min(2, max(0.5, 0.9 (tol/err)^(1/(ord+1)))) for arrays
    h, err as the device controller computes them (correctly rounded pow), on the
    host or on the GPU.  Returns (values, host_pow flags)."""
    lib = load()
    h = np.ascontiguousarray(np.broadcast_to(h, np.shape(err)), dtype=np.float64)
    err = np.ascontiguousarray(err, dtype=np.float64)
    flags = np.zeros(err.size, dtype=np.int32)
    if device:
        out = np.empty_like(err)
        _check(lib.rkcu_step_sizes_device(_ptr(h), _ptr(err), err.size, tol, ord, _ptr(out),
                                          _ptr(flags)), "step_sizes_device")
        return out, flags.astype(bool)
    out = np.empty(err.size)
    f = ctypes.c_int()
    for k, (a, b) in enumerate(zip(h.ravel(), err.ravel())):
        out[k] = lib.rkcu_step_size(a, b, tol, ord, ctypes.byref(f))
        flags[k] = f.value
    return out, flags.astype(bool)


_PREC = {"exact": FP64_EXACT, "fp64": FP64_EXACT, "fma": FP64_FMA, "mixed": MIXED,
         "exact-hwmul": FP64_EXACT_HWMUL}


class Solver:
    """One problem instance on one GPU (an rkcu_solver)."""

    def __init__(self, problem, method="DOPRI54", precision="exact", step_limit=0, device=0,
                 stream=None, wait_timeout_s=10.0, variant=VARIANT_D, block_rows=0, schedule=0,
                 flow_skew=0):
        lib = load()
        self._lib = lib
        self.problem = problem
        self.method = method
        opt = Options()
        lib.rkcu_options_default(ctypes.byref(opt))
        opt.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
        opt.variant = int(variant)
        opt.step_limit = int(step_limit)
        opt.device = int(device)
        opt.stream = stream
        opt.wait_timeout_s = float(wait_timeout_s)
        opt.block_rows = int(block_rows)
        opt.schedule = int(schedule)
        opt.flow_skew = int(flow_skew)
        self._ps = problem.cstruct()
        h = ctypes.c_void_p()
        _check(lib.rkcu_create(ctypes.byref(h), ctypes.byref(self._ps), ctypes.byref(opt)),
               "rkcu_create")
        self._h = h
        if isinstance(method, str):
            _check(lib.rkcu_set_method_by_name(h, method.encode()), f"set_method({method})")
        else:
            self.set_method(**method)

    def set_method(self, A, b, b_hat, c, s, ord, **_):
        A = np.ascontiguousarray(A, dtype=np.float64).reshape(s, s)
        rows = (ctypes.POINTER(ctypes.c_double) * s)(
            *[A[i].ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for i in range(s)])
        self._keep = (A, rows)
        b, b_hat, c = (np.ascontiguousarray(v, dtype=np.float64) for v in (b, b_hat, c))
        _check(self._lib.rkcu_set_method(self._h, rows, _ptr(b), _ptr(b_hat), _ptr(c), s, ord),
               "set_method")

    def solve(self, t0, te, y0, tol):
        """solver(t0, te, y0, y, tol) with host arrays; returns (y, stats dict)."""
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        if y0.size != self.problem.n:
            raise ValueError("y0 has the wrong size")
        y = np.empty_like(y0)
        st = Stats()
        _check(self._lib.rkcu_solve(self._h, t0, te, _ptr(y0), _ptr(y), tol, ctypes.byref(st)),
               "rkcu_solve")
        return y, st.as_dict()

    # device-resident flow --------------------------------------------------
    def begin(self, t0, te, y0, tol, y0_device_ptr=None):
        if y0_device_ptr is not None:
            rc = self._lib.rkcu_begin(self._h, t0, te, ctypes.c_void_p(y0_device_ptr), 1, tol)
        else:
            y0 = np.ascontiguousarray(y0, dtype=np.float64)
            rc = self._lib.rkcu_begin(self._h, t0, te, _ptr(y0), 0, tol)
        _check(rc, "rkcu_begin")

    def advance(self, max_steps):
        _check(self._lib.rkcu_advance(self._h, int(max_steps)), "rkcu_advance")

    def run(self, max_steps):
        """Run up to max_steps attempted steps and wait (rkcu_run)."""
        st = Stats()
        _check(self._lib.rkcu_run(self._h, int(max_steps), ctypes.byref(st)), "rkcu_run")
        return st.as_dict()

    def query(self):
        st = Stats()
        _check(self._lib.rkcu_query(self._h, ctypes.byref(st)), "rkcu_query")
        return st.as_dict()

    def get_y(self, device_ptr=None):
        if device_ptr is not None:
            _check(self._lib.rkcu_get_y(self._h, ctypes.c_void_p(device_ptr), 1), "rkcu_get_y")
            return None
        y = np.empty(self.problem.n)
        _check(self._lib.rkcu_get_y(self._h, _ptr(y), 0), "rkcu_get_y")
        return y

    def set_rhs(self, fn, user=None):
        """The right-hand side of a rhs_problem: "builtin" with user a BRUSS2D-MIX
        or LV-pairs ProblemSpec (rkcu_rhs_builtin), or a Python callable
        fn(t, w_ptr, f_ptr, n, stream) that enqueues f = f(t, w) on the given
        stream and returns 0 (nonzero stops the solve with ERR_RHS)."""
        if isinstance(fn, str) and fn == "builtin":
            ps = user.cstruct()
            self._rhs_keep = (ps, user)
            fptr = ctypes.cast(self._lib.rkcu_rhs_builtin, ctypes.c_void_p)
            uptr = ctypes.cast(ctypes.pointer(ps), ctypes.c_void_p)
            _check(self._lib.rkcu_set_rhs(self._h, fptr, uptr), "rkcu_set_rhs")
            return

        def tramp(t, w, f, n, stream, _user):
            try:
                return int(fn(t, w, f, n, stream) or 0)
            except Exception:  # a Python exception must not cross the C boundary
                import traceback
                traceback.print_exc()
                return 1

        cb = RHS_FN(tramp)
        self._rhs_keep = (cb,)
        _check(self._lib.rkcu_set_rhs(self._h, ctypes.cast(cb, ctypes.c_void_p), None), "rkcu_set_rhs")

    def set_trace(self, capacity, with_y=False):
        """Record the first `capacity` attempted steps after each begin: t, h,
        error max and, with_y, each step's candidate state (rkcu_set_trace)."""
        _check(self._lib.rkcu_set_trace(self._h, int(capacity), 1 if with_y else 0), "rkcu_set_trace")
        self._trace = (int(capacity), bool(with_y))

    def trace(self):
        """The recorded steps: dict of t, h, err arrays and y (steps x n) or None."""
        cap, with_y = getattr(self, "_trace", (0, False))
        t, h, e = np.empty(cap), np.empty(cap), np.empty(cap)
        y = np.empty((cap, self.problem.n)) if with_y else None
        cnt = ctypes.c_int(0)
        _check(self._lib.rkcu_get_trace(self._h, _ptr(t), _ptr(h), _ptr(e),
                                        _ptr(y) if y is not None else None, cap, ctypes.byref(cnt)),
               "rkcu_get_trace")
        k = cnt.value
        return {"t": t[:k], "h": h[:k], "err": e[:k], "y": y[:k] if y is not None else None}

    def inject_wait_timeout(self, extra_arrivals):
        """Test hook: see rkcu_debug_inject_wait_timeout in include/rkcu.h."""
        _check(self._lib.rkcu_debug_inject_wait_timeout(self._h, int(extra_arrivals)),
               "inject_wait_timeout")

    @property
    def stream(self):
        return self._lib.rkcu_stream(self._h)

    @property
    def launches(self):
        return self._lib.rkcu_launch_count(self._h)

    @property
    def device_bytes(self):
        return self._lib.rkcu_device_bytes(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rkcu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def write_dump(path, trace):
    """Write a trace in the reference's DUMP file format (include/tools.h:239-256):
    one line per attempted step, t and h then every component of the candidate
    state, each as %.20e, tab-separated."""
    with open(path, "w") as f:
        f.write(dump_text(trace))


def dump_text(trace):
    """The DUMP file contents of a trace (see write_dump)."""
    ys = trace["y"]
    if ys is None:
        raise ValueError("the trace holds no states (set_trace(..., with_y=True))")
    out = []
    for k in range(len(trace["t"])):
        out.append("%.20e\t%.20e" % (trace["t"][k], trace["h"][k]))
        out.append("".join("\t%.20e" % v for v in ys[k].tolist()))
        out.append("\n")
    return "".join(out)


def footprint(problem, stages=7):
    """Device bytes an instance needs in a Batch arena (admission size)."""
    ps = problem.cstruct()
    return load().rkcu_batch_footprint(ctypes.byref(ps), stages)


class Batch:
    """Many independent solves advanced together on one GPU (rkcu_batch_*).

    add() admits an instance if its footprint fits in the arena (else returns
    None: admission refused, try again after take()); run() advances every
    active instance by up to `sweeps` attempted steps; finished() lists slots
    whose solve is done; take() returns (y, stats, host_id) and frees the slot."""

    def __init__(self, arena_bytes, max_instances, method="DOPRI54", precision="exact",
                 device=0, stream=None, step_limit=0, wait_timeout_s=10.0):
        lib = load()
        self._lib = lib
        opt = Options()
        lib.rkcu_options_default(ctypes.byref(opt))
        opt.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
        opt.step_limit = int(step_limit)
        opt.device = int(device)
        opt.stream = stream
        opt.wait_timeout_s = float(wait_timeout_s)
        h = ctypes.c_void_p()
        _check(lib.rkcu_batch_create(ctypes.byref(h), int(arena_bytes), int(max_instances),
                                     method.encode(), ctypes.byref(opt)), "rkcu_batch_create")
        self._h = h
        self._n = {}

    def add(self, problem, y0, t0, te, tol, host_id=-1):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        ps = problem.cstruct()
        slot = ctypes.c_int(-1)
        rc = self._lib.rkcu_batch_add(self._h, ctypes.byref(ps), t0, te, tol, _ptr(y0),
                                      int(host_id), ctypes.byref(slot))
        if rc == ERR_NOMEM:
            return None
        _check(rc, "rkcu_batch_add")
        self._n[slot.value] = problem.n
        return slot.value

    def run(self, sweeps):
        left = ctypes.c_int()
        _check(self._lib.rkcu_batch_run(self._h, int(sweeps), ctypes.byref(left)), "rkcu_batch_run")
        return left.value

    def finished(self):
        out = []
        buf = np.zeros(1024, dtype=np.int32)
        cnt = ctypes.c_int()
        while True:
            _check(self._lib.rkcu_batch_finished(self._h, _ptr(buf), buf.size, ctypes.byref(cnt)),
                   "rkcu_batch_finished")
            out.extend(int(x) for x in buf[:cnt.value])
            if cnt.value < buf.size:
                return out

    def take(self, slot):
        y = np.empty(self._n[slot])
        st = Stats()
        hid = ctypes.c_longlong()
        _check(self._lib.rkcu_batch_take(self._h, int(slot), _ptr(y), ctypes.byref(st),
                                         ctypes.byref(hid)), "rkcu_batch_take")
        del self._n[slot]
        return y, st.as_dict(), hid.value

    def tune(self, sweeps_per_trial=2):
        best = ctypes.c_double()
        _check(self._lib.rkcu_batch_tune(self._h, int(sweeps_per_trial), ctypes.byref(best)),
               "rkcu_batch_tune")
        return best.value

    def set_tuning(self, threads=256, chunk_pairs=1024, blocks_per_sm=0, use_graph=True):
        _check(self._lib.rkcu_batch_set_tuning(self._h, threads, chunk_pairs, blocks_per_sm,
                                               int(bool(use_graph))), "rkcu_batch_set_tuning")

    def tuning(self):
        t, c, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(self._lib.rkcu_batch_get_tuning(self._h, ctypes.byref(t), ctypes.byref(c),
                                               ctypes.byref(b)), "rkcu_batch_get_tuning")
        return dict(threads=t.value, chunk_pairs=c.value, blocks_per_sm=b.value)

    def info(self):
        a, fb, la = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
        _check(self._lib.rkcu_batch_info(self._h, ctypes.byref(a), ctypes.byref(fb),
                                         ctypes.byref(la)), "rkcu_batch_info")
        return dict(active=a.value, free_bytes=fb.value, launches=la.value)

    @property
    def stream(self):
        return self._lib.rkcu_batch_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.rkcu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def default_tol(method, tol):
    """main.c:47: tol = HAS_EMB_SOL(METHOD) ? TOL : 0.0"""
    return tol if EMBEDDED[method] else 0.0


def solver(t0, te, y0, y, tol, problem, method="DOPRI54", precision="exact", step_limit=0,
           device=0):
    """The reference's solver() contract (include/solver.h:47): integrate y0 from t0
    to te and write the result into y (allocated if None).  Returns (y, stats)."""
    with Solver(problem, method=method, precision=precision, step_limit=step_limit,
                device=device) as s:
        out, st = s.solve(t0, te, y0, tol)
    if y is not None:
        y[...] = out
        out = y
    return out, st

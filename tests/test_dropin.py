r"""The drop-in solver variant (rk_gb300/dropin/D.c): it builds against the
reference's own tree, and on a GPU its stdout equals the reference's.

The reference compares its binaries with log2tab, a state machine over the
stdout lines (log2tab:75-298 of the reference).  With the Perl here and on the
GPU host that script stops every row after the integration interval: its
pattern for the "Initial value" line sits in a double-quoted string, so
"y0\[0\]" reaches the regex engine as the character class "y0[0]" and never
matches.  The rows of a GPU binary and of the reference's own binary are
therefore compared as log2tab prints them (equal, and equally short), and in
full line by line: every line log2tab reads must be the same, apart from the
timings and the solver's name.
"""
import os
import re
import subprocess
import tempfile

import pytest

from conftest import REPO, load_golden

REFERENCE = os.environ.get("RK_REFERENCE", "/root/reference")
LIBDIR = os.path.join(REPO, "rk_gb300", "_lib")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "src")),
                    reason="reference sources not present on this machine")
def test_dropin_links_with_reference_tree(rkcu_lib):
    """D.c compiles with the reference's include/ and links with its main.c, tools.c,
    methods.c, threads.c and bruss2d-mix.c; without a GPU the binary fails loudly."""
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "cuda_bruss2d-mix_D")
        src = [os.path.join(REFERENCE, "src", f) for f in
               ("main.c", "tools.c", "methods.c", "threads.c", "problems/bruss2d-mix.c")]
        subprocess.run(["gcc", "-O2", "-D_GNU_SOURCE", "-D_REENTRANT", "-ffp-contract=off",
                        "-I" + os.path.join(REFERENCE, "include"), "-I" + os.path.join(REPO, "include"),
                        "-DBRUSS_GRID_SIZE=16", "-DSTEP_LIMIT=0", *src,
                        os.path.join(REPO, "rk_gb300", "dropin", "D.c"), "-L" + LIBDIR, "-lrkcu",
                        "-Wl,-rpath," + LIBDIR, "-lpthread", "-lm", "-o", exe],
                       check=True, capture_output=True)
        from conftest import have_gpu
        if not have_gpu():
            p = subprocess.run([exe], capture_output=True, text=True)
            assert p.returncode != 0 and "no usable CUDA device" in p.stderr


def _run(name):
    exe = os.path.join(LIBDIR, name)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    return p.stdout


STAGED = os.path.join(REPO, "baseline", "_ref")
LOG2TAB = os.path.join(STAGED, "log2tab")
# stdout lines log2tab's state machine reads, with the values it copies
LOG2TAB_LINES = ("ODE:", "Grid size:", "Alpha:", "System size:", "Integration interval:",
                 "Initial value:", "Tolerance:", "Lock type:", "Pad size:", "Method:",
                 "Initial step size:", "Number of steps:", "Step limit reached.", "Result:")
P_FLOAT = r"\d+(\.\d+)?e[+-]\d+"


def _log2tab(out):
    p = subprocess.run(["perl", LOG2TAB], input=out, capture_output=True, text=True, timeout=60)
    assert p.returncode == 0, p.stderr
    return p.stdout


def _contract_lines(out):
    return [l for l in out.splitlines() if l.startswith(LOG2TAB_LINES)]


def _compare_with_reference_output(gpu, cpu):
    """Every line log2tab reads is the same, the solver lines parse as log2tab
    parses them, the timing lines have its format; log2tab's own rows agree."""
    assert _contract_lines(gpu) == _contract_lines(cpu)
    for out in (gpu, cpu):
        assert re.search(r"^Solver type: (\S+) embedded Runge-Kutta method", out, re.M)
        assert re.search(r"^Implementation variant: D\b", out, re.M)
        assert re.search(rf"^Kernel time: {P_FLOAT} s \({P_FLOAT} s per step\)", out, re.M)
        assert re.search(rf"^Total time:\s+{P_FLOAT} s", out, re.M)
    assert _log2tab(gpu) == _log2tab(cpu)


have_staged_reference = pytest.mark.skipif(
    not (os.path.exists(LOG2TAB) and os.path.isdir(os.path.join(STAGED, "src"))),
    reason="no copy of the reference sources (baseline/_ref) on this machine")
have_perl = pytest.mark.skipif(subprocess.run(["which", "perl"], capture_output=True).returncode != 0,
                               reason="perl not installed")


@have_staged_reference
@have_perl
@pytest.mark.parametrize("problem,golden", [("bruss2d-mix", "bruss_n250_dopri54_tol1e-6"),
                                            ("lv", "lv_pairs_1000_dopri54")])
def test_standin_runtime_prints_the_reference_contract(problem, golden, rkcu_lib):
    """CPU check of the stand-in runtime (used where the reference tree is absent):
    linked with a stand-in solver that reports the golden step counts, its
    stdout carries every line log2tab reads exactly as the reference's own
    sequential binary prints them for the same configuration."""
    from rk_gb300 import build
    rec = load_golden(golden)
    defs = build.DROPIN["cuda_bruss2d-mix_D" if problem == "bruss2d-mix" else "cuda_lv_D"]
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "fake")
        d = os.path.join(REPO, "rk_gb300", "dropin")
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-I" + os.path.join(d, "compat"),
                        "-I" + os.path.join(REPO, "include"), *["-D" + x for x in defs],
                        f"-DFAKE_ACC={rec['accepted']}", f"-DFAKE_REJ={rec['rejected']}",
                        os.path.join(REPO, "tests", "native", "fake_solver.c"),
                        os.path.join(d, "compat", "runtime.c"), "-L" + LIBDIR, "-lrkcu",
                        "-Wl,-rpath," + LIBDIR, "-lm", "-o", exe], check=True, capture_output=True)
        y0_run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert y0_run.returncode == 0, y0_run.stderr
    cpu = subprocess.run([os.path.join(STAGED, "bin", f"seq_{problem}_D_golden")], capture_output=True,
                         text=True, timeout=600, env=dict(os.environ, NUM_THREADS="1")).stdout
    ref = _contract_lines(cpu)
    got = _contract_lines(y0_run.stdout)
    # the stand-in solver leaves y = y0, so only the Result line differs
    assert [l for l in got if not l.startswith("Result:")] == [l for l in ref if not l.startswith("Result:")]
    assert _log2tab(y0_run.stdout) == _log2tab(cpu)


@pytest.mark.gpu
@have_staged_reference
@have_perl
@pytest.mark.parametrize("problem,golden", [("bruss2d-mix", "bruss_n250_dopri54_tol1e-6"),
                                            ("lv", "lv_pairs_1000_dopri54")])
def test_dropin_with_reference_main_reads_like_the_reference(problem, golden):
    """The drop-in linked with the reference's own main.c, tools.c, methods.c,
    threads.c and problem module (rk_gb300/dropin/Makefile.cuda, built by
    build() from the staged sources): its stdout carries the reference's
    sequential D binary's lines for the same configuration, step counts and
    Result line included, and log2tab makes the same row of both."""
    rec = load_golden(golden)
    gpu = _run(os.path.join("ref", f"cuda_{problem}_D"))
    cpu = subprocess.run([os.path.join(STAGED, "bin", f"seq_{problem}_D_golden")], capture_output=True,
                         text=True, timeout=600, env=dict(os.environ, NUM_THREADS="1")).stdout
    _compare_with_reference_output(gpu, cpu)
    result = [l for l in gpu.splitlines() if l.startswith("Result:")][0]
    assert result == rec["result_line"]


@pytest.mark.gpu
@pytest.mark.parametrize("exe,golden", [("cuda_bruss2d-mix_D", "bruss_n250_dopri54_tol1e-6"),
                                        ("cuda_lv_D", "lv_pairs_1000_dopri54")])
def test_dropin_stdout_equals_reference(exe, golden):
    rec = load_golden(golden)
    out = _run(exe)
    m = re.search(r"Number of steps: (\d+) \((\d+) accepted, (\d+) rejected\)", out)
    assert m and tuple(map(int, m.groups())) == (rec["steps"], rec["accepted"], rec["rejected"])
    result = [l for l in out.splitlines() if l.startswith("Result:")][0]
    assert result == rec["result_line"]
    if os.path.exists(LOG2TAB) and subprocess.run(["which", "perl"], capture_output=True).returncode == 0:
        assert re.search(r"^Lock type: \w+$", out, re.M) and re.search(r"^Pad size: \d+$", out, re.M)
        assert _log2tab(out).count(",") >= 5

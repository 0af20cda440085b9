"""The drop-in solver variant (rk_gb300/dropin/D.c): it builds against the
reference's own tree, and on a GPU its stdout equals the reference's."""
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

"""The batch arena's free list (rk_gb300/csrc/rkcu_arena.h): first-fit
allocation and coalescing on release, against a byte map of the arena over
random allocate/release sequences (tests/native/arena_check.cpp)."""
import os
import subprocess
import tempfile

from conftest import REPO


def test_arena_first_fit_and_coalescing():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "arena")
        subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(REPO, "rk_gb300", "csrc"),
                        os.path.join(REPO, "tests", "native", "arena_check.cpp"), "-o", exe], check=True)
        for seed in (1, 2):
            p = subprocess.run([exe, "3000", str(seed)], capture_output=True, text=True)
            assert p.returncode == 0, p.stdout

"""Software binary64 multiply/add (rk_gb300/csrc/rkcu_softfp64.cuh): bit-identical
to IEEE round-to-nearest arithmetic, on the host (CPU test) and on the device
against the FP64 pipe (GPU test)."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "rk_gb300", "csrc")
NATIVE = os.path.join(REPO, "tests", "native")


def test_softfp64_host_bit_exact():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "sfp")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(NATIVE, "softfp64_check.cpp"), "-o", exe], check=True)
        for seed in (1, 2):
            p = subprocess.run([exe, "5000000", str(seed)], capture_output=True, text=True)
            assert p.returncode == 0, p.stdout


@pytest.mark.gpu
def test_softfp64_device_bit_exact():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "sfpg")
        subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-I" + CSRC, os.path.join(NATIVE, "softfp64_check.cu"), "-o", exe], check=True)
        p = subprocess.run([exe, str(1 << 28), "3"], capture_output=True, text=True)
        assert p.returncode == 0, p.stdout + p.stderr

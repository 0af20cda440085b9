"""Double-float arithmetic and the fixed-point Laplacian of the mixed form's
stage 0 (rk_gb300/csrc/rkcu_dfloat.cuh): accuracy against long double on the
host (CPU test), and the same bits on the device as on the host (GPU test)."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import REPO

CSRC = os.path.join(REPO, "rk_gb300", "csrc")
NATIVE = os.path.join(REPO, "tests", "native")


def test_dfloat_host_accuracy():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "dfc")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(NATIVE, "dfloat_check.cpp"), "-o", exe], check=True)
        for seed in (1, 2):
            p = subprocess.run([exe, "2000000", str(seed)], capture_output=True, text=True)
            assert p.returncode == 0, p.stdout
            assert "refused 0" in p.stdout


@pytest.mark.gpu
def test_dfloat_device_matches_host():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "dfcg")
        subprocess.run([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-Xcompiler", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(NATIVE, "dfloat_check.cu"), "-o", exe], check=True)
        p = subprocess.run([exe, str(1 << 20), "5"], capture_output=True, text=True)
        assert p.returncode == 0, p.stdout + p.stderr

"""Shared test setup: the `gpu` marker, paths, golden fixtures, built libraries."""
import glob
import json
import os
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)
ORACLE_DIR = os.path.join(REPO, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def all_golden():
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.json"))):
        with open(p) as f:
            out.append(json.load(f))
    return out


def golden_y(rec):
    """(indices, values) of the stored final state components."""
    if "y_hex" in rec:
        v = np.array([float.fromhex(x) for x in rec["y_hex"]])
        return np.arange(v.size), v
    st = rec["y_sample"]["stride"]
    v = np.array([float.fromhex(x) for x in rec["y_sample"]["values"]])
    return np.arange(0, rec["n"], st)[: v.size], v


def golden_y0(rec):
    import rk_oracle
    if rec["problem"] == "bruss2d-mix":
        return rk_oracle.bruss_start(rec["grid_n"])
    return rk_oracle.lv_pairs_start(rec["n"])


@pytest.fixture(scope="session")
def oracle():
    import rk_oracle
    rk_oracle.build()
    rk_oracle.load()
    return rk_oracle


@pytest.fixture(scope="session")
def rkcu_lib():
    """librkcu.so, built in tree if missing (nvcc cross-compiles without a GPU)."""
    import rk_gb300
    if not os.path.exists(rk_gb300.LIB_PATH):
        from rk_gb300 import build
        build.build_cuda()
    return rk_gb300.load()


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

"""Build the rkcu CUDA library (sm_103a) and the CPU oracle, in tree.

    python -m rk_gb300.build            # librkcu.so + oracle
    python -m rk_gb300.build --verbose  # also print -Xptxas -v resource usage

Outputs (git-ignored): rk_gb300/_lib/librkcu.so, oracle/_build/librk_oracle.so,
rk_gb300/_lib/cuda_bruss2d-mix_D (drop-in driver binary).
Each translation unit is compiled in parallel with one -gencode, so a build
takes well under a minute on the GPU host as well as here.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")

CU_SOURCES = ["rkcu_api.cu", "rkcu_plain.cu", "rkcu_methods.cu", "rkcu_noalloc.cu", "rkcu_mixed.cu",
              "rkcu_batch.cu", "rkcu_batch_api.cu", "rkcu_lowstorage.cu", "rkcu_general.cu"]
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build_cuda(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    flags = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
             "-I" + INCLUDE, "-I" + CSRC, "--expt-relaxed-constexpr"]
    if verbose:
        flags.append("-Xptxas=-v")
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        jobs.append((obj, [nvcc(), *flags, "-c", os.path.join(CSRC, src), "-o", obj]))
    outs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(lambda j: _run(j[1]), jobs):
            outs.append(out)
    lib = os.path.join(LIBDIR, "librkcu.so")
    tmp = lib + ".tmp"
    _run([nvcc(), GENCODE, "-shared", "-o", tmp, *[j[0] for j in jobs], "-lcudart"])
    os.replace(tmp, lib)
    if verbose:
        sys.stdout.write("".join(outs))
    return lib


def build_oracle():
    _run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "oracle"])
    return os.path.join(REPO, "oracle", "_build", "librk_oracle.so")


# Drop-in driver binaries (bin/<family>_<problem>_<variant> naming of the
# reference's Makefile): the drop-in D.c + the stand-in runtime, one
# configuration each, as the reference builds one binary per configuration.
DROPIN = {
    "cuda_bruss2d-mix_D": ["BRUSS_GRID_SIZE=250", "BRUSS_ALPHA=2E-3", "METHOD=DOPRI54", "TOL=1E-6",
                           "T_END=0.5", "STEP_LIMIT=0"],
    "cuda_lv_D": ["RKCU_PROBLEM_LV", "LV_COUNT=1000", "METHOD=DOPRI54", "TOL=1E-6", "T_END=10.0",
                  "STEP_LIMIT=0"],
}


def build_dropin():
    d = os.path.join(PKG, "dropin")
    cc = shutil.which("gcc") or "cc"
    out = []
    for name, defs in DROPIN.items():
        exe = os.path.join(LIBDIR, name)
        _run([cc, "-O2", "-std=gnu11", "-Wall", "-ffp-contract=off", "-I" + os.path.join(d, "compat"),
              "-I" + INCLUDE, *["-D" + x for x in defs], os.path.join(d, "D.c"),
              os.path.join(d, "compat", "runtime.c"), "-L" + LIBDIR, "-lrkcu",
              "-Wl,-rpath,$ORIGIN", "-lm", "-o", exe])
        out.append(exe)
    return out


# The same drop-in linked with the reference's own main.c, tools.c, methods.c,
# threads.c and problem module (rk_gb300/dropin/Makefile.cuda), when a copy of
# the reference sources is at hand (RK_REFERENCE, or the staged copy in
# baseline/_ref), with the configurations of two golden fixtures; and the
# reference's sequential D binaries of the same configurations, so that both
# rows can be read by the reference's log2tab side by side.
REF_DROPIN = {
    "bruss2d-mix": ["BRUSS_GRID_SIZE=250", "BRUSS_ALPHA=2E-3", "METHOD=DOPRI54", "TOL=1E-6",
                    "T_END=0.5", "STEP_LIMIT=0"],
    "lv": ["LV_COUNT=1000", "METHOD=DOPRI54", "TOL=1E-6", "T_END=10.0", "STEP_LIMIT=0"],
}
REF_DROPIN_DIR = os.path.join(LIBDIR, "ref")


def build_dropin_reference():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import stage_reference
    root = stage_reference.source_root()
    if not root:
        return []
    out = []
    for problem, defs in REF_DROPIN.items():
        _run(["make", "-s", "-f", os.path.join(PKG, "dropin", "Makefile.cuda"), "cuda",
              f"REF={root}", f"BINDIR={REF_DROPIN_DIR}", f"CUDA_PROBLEMS={problem}",
              "CUDA_EXTRA_CFLAGS=-ffp-contract=off",
              "DEFINES=" + " ".join(defs)])
        out.append(os.path.join(REF_DROPIN_DIR, f"cuda_{problem}_D"))
        d = dict(x.split("=") for x in defs)
        d["PROBLEM"] = problem
        out.append(stage_reference.build_solver("seq/D", d, name=f"seq_{problem}_D_golden",
                                                contract=False))
    return out


def build_all(verbose=False):
    lib = build_cuda(verbose)
    orc = build_oracle()
    build_dropin()
    return lib, orc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build_all(a.verbose))


if __name__ == "__main__":
    main()

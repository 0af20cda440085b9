"""Stage the reference's sources into baseline/_ref/ and compile its CPU solvers.

Test and baseline infrastructure, not part of the product.  The reference is a
C code without a package to install; its CPU solvers are compiled from its own
source files, which must therefore travel to a machine that has no copy of the
reference tree.  stage() copies the files the CPU baseline, the drop-in
checks and the log2tab checks compile or run -- include/*.h, src/*.c,
src/problems/*.c, src/impl/{seq,pthreads}/*.c and the log2tab script -- from
the reference tree (environment variable RK_REFERENCE) into baseline/_ref/,
which git ignores.  build_solver() compiles one reference binary from the staged
copy (or from the tree itself) with the reference's own compiler flags
(Makefile:45-53: -I include -D_REENTRANT -Wall -O3 -g -D_GNU_SOURCE, MPI off)
plus the configuration's -D defines, exactly as the reference's Makefile
builds bin/<family>_<problem>_<variant>; nothing of the reference is changed.
"""
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
STAGED = os.path.join(REPO, "baseline", "_ref")
BIN = os.path.join(STAGED, "bin")

PATTERNS = ["include/*.h", "src/*.c", "src/problems/*.c", "src/impl/seq/*.c",
            "src/impl/pthreads/*.c", "log2tab"]

# the reference Makefile's CFLAGS (Makefile:45) with HAVE_MPI=no, and LDFLAGS (Makefile:51)
REF_CFLAGS = ["-D_REENTRANT", "-Wall", "-O3", "-g", "-D_GNU_SOURCE"]
REF_LDFLAGS = ["-lpthread", "-lm"]


def reference_tree():
    """The reference tree named by RK_REFERENCE, if present here."""
    root = os.environ.get("RK_REFERENCE", "/root/reference")
    return root if os.path.isdir(os.path.join(root, "src")) else None


def source_root():
    """Where reference sources can be compiled from: the tree itself, else the staged copy."""
    tree = reference_tree()
    if tree:
        return tree
    return STAGED if os.path.isdir(os.path.join(STAGED, "src")) else None


def stage():
    """Copy the needed reference files into baseline/_ref/ (no-op without a reference tree)."""
    tree = reference_tree()
    if not tree:
        return None
    for pat in PATTERNS:
        for src in glob.glob(os.path.join(tree, pat)):
            dst = os.path.join(STAGED, os.path.relpath(src, tree))
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            shutil.copy2(src, dst)
    return STAGED


def build_solver(variant, defines, name=None, root=None, contract=True):
    """Compile bin/<name> from the reference's main.c, tools.c, methods.c, threads.c,
    problems/bruss2d-mix.c (or lv.c: defines containing "PROBLEM=lv") and
    src/impl/<variant>.c.  contract=False adds -ffp-contract=off: the
    reference's flags leave multiply-add contraction to the compiler, which
    fuses on aarch64 and not on x86-64, so only without contraction are its
    results the same on both (and equal to the golden fixtures).  Returns the
    executable's path, or None without sources."""
    root = root or source_root()
    if not root:
        return None
    defines = dict(defines)
    problem = defines.pop("PROBLEM", "bruss2d-mix")
    name = name or f"{variant.replace('/', '_')}_{problem}"
    os.makedirs(BIN, exist_ok=True)
    exe = os.path.join(BIN, name)
    src = [os.path.join(root, "src", f) for f in ("main.c", "tools.c", "methods.c", "threads.c")]
    src += [os.path.join(root, "src", "problems", problem + ".c"),
            os.path.join(root, "src", "impl", variant + ".c")]
    cmd = ["gcc", "-I" + os.path.join(root, "include"), *REF_CFLAGS,
           *([] if contract else ["-ffp-contract=off"]),
           *[f"-D{k}={v}" for k, v in defines.items()], "-o", exe, *src, *REF_LDFLAGS]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


if __name__ == "__main__":
    print(stage())

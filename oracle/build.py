"""Build recipe for the ORACLE shared library (test infrastructure only).

Compiles the plain-C FP64 restatement of SEM2DPACK's initialisation and
time step into ``oracle/_build/libsem2d_oracle.so``.  FMA contraction is
disabled so that x86-64 and aarch64 hosts evaluate the same expressions.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["oc_gll.c", "oc_setup.c", "oc_step.c"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsem2d_oracle.so")


def build(force=False, verbose=False):
    """Compile the oracle library if a source is newer than it; return its path."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "sem2d_oracle.h"),
                   os.path.join(HERE, "..", "include", "sem2d_host.h"),
                   os.path.join(HERE, "..", "include", "sem2d_gpu.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-Wno-unused-variable", "-o", tmp] + srcs + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/tfhe_oracle.cpp into oracle/_build/libtfhe_oracle.so with
g++.  Portable flags only (the same file builds on x86_64 and aarch64):
no -march=native, and -ffp-contract=off so that both machines round every
floating-point operation the same way.

Also compiles oracle/tfhe_cpu_fast.cpp (the faster CPU gate bootstrap that
bench.py times beside the oracle) into oracle/_build/libtfhe_cpu_fast.so,
with the compiler's default contraction (FMA where the machine has it):
it is timed, not used as a checker.

    python oracle/build_oracle.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtfhe_oracle.so")
SRC = os.path.join(HERE, "tfhe_oracle.cpp")
HDR = os.path.join(HERE, "tfhe_oracle.h")
FAST_LIB = os.path.join(BUILD, "libtfhe_cpu_fast.so")
FAST_SRC = os.path.join(HERE, "tfhe_cpu_fast.cpp")


def _compile(lib, src, extra, force, verbose):
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(src), os.path.getmtime(HDR))):
        return lib
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp"] + extra + [
        "-Wall", "-Wno-unknown-pragmas", src, "-o", lib + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build(force=False, verbose=False):
    """Both libraries; returns the oracle's path."""
    os.makedirs(BUILD, exist_ok=True)
    _compile(FAST_LIB, FAST_SRC, [], force, verbose)
    return _compile(LIB, SRC, ["-ffp-contract=off"], force, verbose)


def build_fast(force=False, verbose=False):
    """The faster CPU gate bootstrap only; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    return _compile(FAST_LIB, FAST_SRC, [], force, verbose)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

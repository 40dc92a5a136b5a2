"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/tfhe_oracle.cpp into oracle/_build/libtfhe_oracle.so with
g++.  Portable flags only (the same file builds on x86_64 and aarch64):
no -march=native, and -ffp-contract=off so that both machines round every
floating-point operation the same way.

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


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas",
           SRC, "-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

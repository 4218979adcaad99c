"""Build recipe for the oracle library (test infrastructure only).

liboracle.so is the CPU restatement in sfo.cpp, compiled with
-ffp-contract=off so that every float operation rounds once, as the
reference's source states it.  Output: oracle/liboracle.so (git-ignored).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "sfo.cpp")]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources + [os.path.join(HERE, "sfo.h")])


def build(force=False, verbose=False):
    if not force and not _stale(LIB, SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-fPIC", "-shared", "-Wall", "-o", LIB + ".tmp"] + SRC
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)

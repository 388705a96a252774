"""Build recipe for the oracle (test infrastructure).

Compiles oracle/fargo_oracle.cpp into oracle/_build/libfargo_oracle.so with
g++ -O2 -fopenmp -ffp-contract=off (no fused multiply-add, so the arithmetic is
the plain IEEE sequence written in the source on x86_64 and aarch64 alike).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfargo_oracle.so")
SRC = [os.path.join(HERE, "fargo_oracle.cpp")]
DEPS = SRC + [os.path.join(HERE, "fft_ref.h"),
              os.path.join(HERE, "..", "include", "fargo_gb300.h")]

CXXFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            "-fno-fast-math", "-std=c++17"]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in DEPS)


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++"] + CXXFLAGS + SRC + ["-o", LIB + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

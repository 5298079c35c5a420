"""Build recipe for the oracle (test infrastructure only).

Compiles dana_oracle.cpp and oracle_gen.cpp into oracle/_build/liboracle.so with the flags that
keep the reference's floating-point evaluation order: no FMA contraction
(-ffp-contract=off) and no value-changing optimisation (no -ffast-math).
The same source and flags give identical results on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "dana_oracle.cpp"), os.path.join(HERE, "oracle_gen.cpp")]
DEPS = SRC + [os.path.join(HERE, "oracle.h"),
              os.path.join(HERE, "..", "include", "dml.h"),
              os.path.join(HERE, "..", "include", "dml_rng.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force=False, verbose=False):
    """Compile liboracle.so if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-Wall", "-o", LIB + ".tmp"] + SRC
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

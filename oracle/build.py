"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/pgdg_oracle.cpp and oracle/oracle_case.cpp with g++ into oracle/_build/liboracle.so.
-ffp-contract=off keeps every expression in written order with one rounding per
operation on both x86_64 and aarch64 (where GCC would otherwise contract into FMA).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRCS = [os.path.join(HERE, "pgdg_oracle.cpp"), os.path.join(HERE, "oracle_case.cpp")]
DEPS = SRCS + [os.path.join(HERE, "oracle_math.h"), os.path.join(HERE, "pgdg_oracle.h"),
               os.path.join(HERE, "..", "include", "pgdg_types.h")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + SRCS
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

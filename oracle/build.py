"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/pgdg_oracle.cpp and oracle/oracle_case.cpp with g++ into
oracle/_build/liboracle.so (two materials) and liboracle_f3.so (-DPO_NFLD=3, the
three-material instance).
-ffp-contract=off keeps every expression in written order with one rounding per
operation on both x86_64 and aarch64 (where GCC would otherwise contract into FMA).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
SRCS = [os.path.join(HERE, "pgdg_oracle.cpp"), os.path.join(HERE, "oracle_case.cpp")]
DEPS = SRCS + [os.path.join(HERE, "oracle_math.h"), os.path.join(HERE, "pgdg_oracle.h"),
               os.path.join(HERE, "..", "include", "pgdg_types.h")]


def lib_path(nfld=2):
    """The oracle library of a material count: two (every workload) or three."""
    return os.path.join(OUT_DIR, "liboracle.so" if nfld == 2 else f"liboracle_f{nfld}.so")


LIB = lib_path(2)


def build(force=False, verbose=False):
    """Builds the oracle for two and for three materials (in parallel); returns
    the two-material library's path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    procs = []
    for nfld in (2, 3):
        lib = lib_path(nfld)
        if not force and os.path.exists(lib):
            t = os.path.getmtime(lib)
            if all(os.path.getmtime(d) <= t for d in DEPS):
                continue
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
               f"-DPO_NFLD={nfld}", "-o", lib + ".tmp"] + SRCS
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd), lib))
    for pr, lib in procs:
        if pr.wait() != 0:
            raise subprocess.CalledProcessError(pr.returncode, "g++ (oracle)")
        os.replace(lib + ".tmp", lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

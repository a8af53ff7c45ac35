"""Build of libpgdg_gpu.so for sm_103a (in tree, nvcc only, no cmake).

Each CUDA translation unit is compiled in parallel to an object, then linked into
pgdg_p2_gb300/_build/libpgdg_gpu.so (two materials) and, from the same sources
with -DPGDG_NFLD=3, pgdg_p2_gb300/_build_f3/libpgdg_gpu_f3.so (the 2D
three-material instance; FldNum is a compile-time constant, as in the reference).  k_particles.cu (split/merge/binning) is
compiled with -fmad=false so its FP64 arithmetic matches the oracle bit for bit.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpgdg_gpu.so")
INC = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (source, object tag, extra flags): the grid, G2P and output kernels are compiled twice,
# once with FMA contraction (mixed and FP64_FMA paths) and once without
# (-DPGDG_EXACT_TU: the exact-order FP64 path)
CU = [("k_particles.cu", "k_particles", ["-fmad=false"]),
      ("k_grid.cu", "k_grid", []),
      ("k_grid.cu", "k_grid_x", ["-fmad=false", "-DPGDG_EXACT_TU"]),
      ("k_g2p.cu", "k_g2p", []),
      ("k_g2p.cu", "k_g2p_x", ["-fmad=false", "-DPGDG_EXACT_TU"]),
      ("k_mlp.cu", "k_mlp", ["-fmad=false"]),
      ("k_xfer.cu", "k_xfer", []),
      ("k_mlp_tc.cu", "k_mlp_tc", []),
      ("k_peak.cu", "k_peak", []),
      ("k_case.cu", "k_case", ["-fmad=false"]),
      ("k_output.cu", "k_output", []),
      ("k_output.cu", "k_output_x", ["-fmad=false", "-DPGDG_EXACT_TU"]),
      ("capi.cu", "capi", [])]
CPP = ["case_builder.cpp", "plt_writer.cpp"]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    d = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    d += [os.path.join(INC, f) for f in os.listdir(INC)]
    return d


def lib_path(nfld=2):
    """The library of a material count: libpgdg_gpu.so (two materials, every 2D and
    3D workload) or libpgdg_gpu_f3.so (-DPGDG_NFLD=3, the 2D three-material case)."""
    return LIB if nfld == 2 else os.path.join(HERE, f"_build_f{nfld}", f"libpgdg_gpu_f{nfld}.so")


def build(force=False, verbose=False):
    """Builds both libraries (their translation units compiled in parallel);
    returns the two-material library's path."""
    nvcc = _nvcc()
    deps = _deps()
    jobs, links = [], []
    for nfld in (2, 3):
        lib = lib_path(nfld)
        out = os.path.dirname(lib)
        os.makedirs(out, exist_ok=True)
        if not force and os.path.exists(lib):
            t = os.path.getmtime(lib)
            if all(os.path.getmtime(x) <= t for x in deps):
                continue
        nf = [] if nfld == 2 else [f"-DPGDG_NFLD={nfld}"]
        objs = []
        for f, tag, extra in CU:
            obj = os.path.join(out, tag + ".o")
            cmd = [nvcc] + ARCH + extra + nf + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler",
                                                "-fPIC,-ffp-contract=off", "-I", INC, "-c",
                                                os.path.join(CSRC, f), "-o", obj]
            jobs.append((cmd, obj))
            objs.append(obj)
        for f in CPP:
            obj = os.path.join(out, f + ".o")
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INC, "-c",
                   os.path.join(CSRC, f), "-o", obj]
            jobs.append((cmd, obj))
            objs.append(obj)
        links.append((lib, objs))

    def run(job):
        cmd, obj = job
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    for lib, objs in links:
        tmp = lib + ".tmp"
        # every symbol resolved at link time (a missing instantiation fails here, not at load)
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-Xlinker", "--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

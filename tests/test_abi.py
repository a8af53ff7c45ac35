"""The C-ABI library loads without a GPU and exports every symbol its headers
declare; the ctypes layouts match the C structures."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from pgdg_p2_gb300 import abi, mpm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix):
    txt = open(os.path.join(ROOT, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"\w+)\s*\(", txt)))


def test_gpu_library_exports_header_symbols():
    lib = mpm.lib()
    names = declared("include/pgdg.h", "pgdg_")
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports_header_symbols():
    from oracle import oracle as O
    lib = O.lib()
    names = declared("oracle/pgdg_oracle.h", "po_")
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_create_fails_loudly_without_gpu():
    # on a machine without a GPU the context refuses to exist (no CPU fallback)
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    cs = mpm.case_setup(1, (8, 4))
    with pytest.raises(abi.PgdgError):
        mpm.MPM(cs)


def test_struct_layouts_match_c():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "pgdg_types.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(pgdg_case), sizeof(pgdg_particles), sizeof(pgdg_cells),
         sizeof(pgdg_stats), offsetof(pgdg_case, probe), offsetof(pgdg_case, cfl), offsetof(pgdg_cells, dcoef));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    exp = [ctypes.sizeof(abi.pgdg_case), ctypes.sizeof(abi.pgdg_particles), ctypes.sizeof(abi.pgdg_cells),
           ctypes.sizeof(abi.pgdg_stats), abi.pgdg_case.probe.offset, abi.pgdg_case.cfl.offset,
           abi.pgdg_cells.dcoef.offset]
    assert out == exp


def test_create_rejects_rows_beyond_16_bit_offsets():
    # the mixed and FP64_FMA shifting kernel sorts each row of cells along the
    # last axis with 16-bit cell offsets: a longer last axis is refused before
    # any GPU call (so this runs without a GPU); the exact path has no row sort
    import ctypes as C
    from pgdg_p2_gb300.abi import PREC_MIXED
    lib = mpm.lib()
    for dim, grid in ((2, (4, 65536)), (3, (2, 2, 70000))):
        cs = mpm.case_setup(1 if dim == 2 else 3, (8, 4) if dim == 2 else (8, 4, 4))
        for d in range(dim):
            cs.ncell[d] = grid[d]
        h = C.c_void_p()
        for prec in (PREC_MIXED, 2):
            assert lib.pgdg_create(C.byref(cs), prec, 0, C.byref(h)) == -1
        cs.ncell[dim - 1] = 0
        assert lib.pgdg_create(C.byref(cs), 0, 0, C.byref(h)) == -1

"""ctypes loader of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.  It wraps oracle/pgdg_oracle.h with the same method names
the device wrapper (pgdg_p2_gb300.mpm.MPM) exposes, so a test can run one call on
both and compare.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from pgdg_p2_gb300.abi import (Cells, Particles, check, pgdg_case, pgdg_cells,  # noqa: E402
                               pgdg_particles, pgdg_stats)
from oracle import build as _build  # noqa: E402

_libs = {}


def lib(nfld=2):
    """The oracle library of a material count (2, or 3 for the three-material case)."""
    if nfld not in _libs:
        _build.build()
        L = C.CDLL(_build.lib_path(nfld))
        P = C.POINTER
        vp = C.c_void_p
        L.po_create.argtypes = [P(pgdg_case), P(vp)]
        for name in ("po_destroy", "po_used_state_update", "po_bin_particles", "po_split_particle_fast",
                     "po_merge_particle_fast", "po_refresh_membership", "po_refresh_neighbors",
                     "po_mls_p2g", "po_calculate_limiter", "po_grid_acceleration"):
            getattr(L, name).argtypes = [vp]
        L.po_upload_particles.argtypes = [vp, P(pgdg_particles)]
        L.po_download_particles.argtypes = [vp, P(pgdg_particles)]
        L.po_num_particles.argtypes = [vp, P(C.c_int64)]
        L.po_upload_cells.argtypes = [vp, P(pgdg_cells)]
        L.po_download_cells.argtypes = [vp, P(pgdg_cells)]
        L.po_upload_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64)]
        L.po_download_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64), C.c_int64, P(C.c_int64)]
        L.po_download_cell_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64), C.c_int64, P(C.c_int64)]
        L.po_set_dt.argtypes = [vp, C.c_double]
        L.po_set_iterate.argtypes = [vp, C.c_int64]
        L.po_set_max_v.argtypes = [vp, C.c_double]
        L.po_get_stats.argtypes = [vp, P(pgdg_stats)]
        L.po_set_timestep.argtypes = [vp, P(C.c_double), P(C.c_double)]
        L.po_update_grid.argtypes = [vp, C.c_int]
        L.po_update_particle.argtypes = [vp, C.c_int]
        L.po_run_step.argtypes = [vp, C.c_int64]
        L.po_advance.argtypes = [vp, C.c_int]
        L.po_totals.argtypes = [vp, P(C.c_double)]
        L.po_output_point.argtypes = [vp, P(C.c_double)]
        L.po_output_plt.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.po_set_threads.argtypes = [C.c_int]
        L.po_mgfm_batched.argtypes = [P(C.c_double), P(C.c_int8), P(C.c_double), P(C.c_double), C.c_int,
                                      P(C.c_double), P(C.c_double), P(C.c_int32), C.c_int64]
        L.po_root_d.argtypes = [C.c_double, C.c_int]
        L.po_root_d.restype = C.c_double
        L.po_case_setup.argtypes = [C.c_int, P(C.c_int32), P(pgdg_case)]
        L.po_case_num_particles.argtypes = [P(pgdg_case)]
        L.po_case_num_particles.restype = C.c_int64
        L.po_case_particles.argtypes = [P(pgdg_case), C.c_int, C.c_uint64, P(pgdg_particles)]
        L.po_case_cells.argtypes = [P(pgdg_case), P(pgdg_cells)]
        _libs[nfld] = L
    return _libs[nfld]


def set_threads(n):
    lib().po_set_threads(int(n))


def case_setup(config_id, ncell=None):
    """The oracle's own pgdg_case of workload config_id (grid override ncell)."""
    cs = pgdg_case()
    nc = (C.c_int32 * 3)(*(ncell or (0, 0, 0)))
    check(lib().po_case_setup(int(config_id), nc, C.byref(cs)), "po_case_setup")
    return cs


def case_particles(cs, config_id, seed=0):
    p = Particles(lib().po_case_num_particles(C.byref(cs)), cs.dim)
    check(lib().po_case_particles(C.byref(cs), int(config_id), int(seed), C.byref(p.view())), "po_case_particles")
    return p


def case_cells(cs):
    c = Cells(cs.ncells, cs.dim, nfld=cs.nfld)
    check(lib().po_case_cells(C.byref(cs), C.byref(c.view())), "po_case_cells")
    return c


def make_case(config_id, ncell=None, seed=0):
    """(case, particles, cells) built by the oracle alone, without the GPU library."""
    cs = case_setup(config_id, ncell)
    return cs, case_particles(cs, config_id, seed), case_cells(cs)


class Oracle:
    """FP64 serial restatement of the reference path (see oracle/pgdg_oracle.cpp)."""

    def __init__(self, cs: pgdg_case):
        self.cs = cs
        self.dim = cs.dim
        self.h = C.c_void_p()
        self._L = lib(cs.nfld)
        check(self._L.po_create(C.byref(cs), C.byref(self.h)), "po_create")

    def __del__(self):
        if getattr(self, "h", None) and getattr(self, "_L", None) is not None:
            self._L.po_destroy(self.h)
            self.h = None

    # ---- state exchange ----
    def upload_particles(self, p: Particles):
        v = p.view()
        v.n = p.n
        check(self._L.po_upload_particles(self.h, C.byref(v)), "upload_particles")

    def num_particles(self):
        n = C.c_int64()
        self._L.po_num_particles(self.h, C.byref(n))
        return n.value

    def download_particles(self):
        n = self.num_particles()
        p = Particles(n, self.dim)
        v = p.view()
        check(self._L.po_download_particles(self.h, C.byref(v)), "download_particles")
        return p

    def upload_cells(self, c: Cells):
        check(self._L.po_upload_cells(self.h, C.byref(c.view())), "upload_cells")

    def download_cells(self):
        c = Cells(self.cs.ncells, self.dim, nfld=self.cs.nfld)
        check(self._L.po_download_cells(self.h, C.byref(c.view())), "download_cells")
        return c

    def _csr(self, fn, nrow):
        tot = C.c_int64()
        off = np.zeros(nrow + 1, np.int64)
        fn(self.h, off.ctypes.data_as(C.POINTER(C.c_int64)), None, 0, C.byref(tot))
        ent = np.zeros(max(tot.value, 1), np.int64)
        check(fn(self.h, off.ctypes.data_as(C.POINTER(C.c_int64)), ent.ctypes.data_as(C.POINTER(C.c_int64)),
                 ent.size, C.byref(tot)), "download csr")
        return off, ent[: tot.value]

    def download_lists(self):
        return self._csr(self._L.po_download_lists, self.num_particles())

    def download_cell_lists(self):
        return self._csr(self._L.po_download_cell_lists, self.cs.ncells)

    def upload_lists(self, off, ent):
        off = np.ascontiguousarray(off, np.int64)
        ent = np.ascontiguousarray(ent if len(ent) else np.zeros(1, np.int64), np.int64)
        check(self._L.po_upload_lists(self.h, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                    ent.ctypes.data_as(C.POINTER(C.c_int64))), "upload_lists")

    def set_dt(self, dt):
        self._L.po_set_dt(self.h, float(dt))

    def set_iterate(self, n):
        self._L.po_set_iterate(self.h, int(n))

    def set_max_v(self, mv):
        self._L.po_set_max_v(self.h, float(mv))

    def stats(self):
        s = pgdg_stats()
        self._L.po_get_stats(self.h, C.byref(s))
        return s.to_dict()

    # ---- reference methods ----
    def Set_timestep(self):
        dt, mv = C.c_double(), C.c_double()
        self._L.po_set_timestep(self.h, C.byref(dt), C.byref(mv))
        return dt.value, mv.value

    def Used_state_update(self):
        self._L.po_used_state_update(self.h)

    def Map_the_particle_to_tree(self):
        self._L.po_bin_particles(self.h)

    def Split_particle_fast(self):
        self._L.po_split_particle_fast(self.h)

    def Merge_particle_fast(self):
        self._L.po_merge_particle_fast(self.h)

    def Refresh_membership(self):
        self._L.po_refresh_membership(self.h)

    def Refresh_neighbors(self):
        self._L.po_refresh_neighbors(self.h)

    def MLS_P2G(self):
        self._L.po_mls_p2g(self.h)

    def Calculate_limiter(self):
        self._L.po_calculate_limiter(self.h)

    def Grid_acceleration(self):
        self._L.po_grid_acceleration(self.h)

    def Update_grid(self, md):
        self._L.po_update_grid(self.h, int(md))

    def Update_particle(self, md):
        self._L.po_update_particle(self.h, int(md))

    def MPM_run_simulation(self, n):
        self._L.po_run_step(self.h, int(n))

    def advance(self, nsteps):
        self._L.po_advance(self.h, int(nsteps))

    def output_point(self):
        out = np.zeros(5)
        self._L.po_output_point(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def output_plt(self, particle_path=None, cell_path=None):
        """Output_plt_file: the particle Tecplot binary and the cell table."""
        enc = (lambda p: str(p).encode() if p is not None else None)
        rc = self._L.po_output_plt(self.h, enc(particle_path), enc(cell_path))
        if rc != 0:
            raise RuntimeError(f"po_output_plt failed ({rc})")

    def totals(self):
        """Particle mass per phase, particle energy, cell mass per phase, cell energy."""
        out = np.zeros(2 * self.cs.nfld + 2)
        self._L.po_totals(self.h, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out


def mgfm_batched(in6, mat2, gam, pinf, variant=0, seed=None):
    in6 = np.ascontiguousarray(in6, np.float64)
    mat2 = np.ascontiguousarray(mat2, np.int8)
    gam = np.ascontiguousarray(gam, np.float64)
    pinf = np.ascontiguousarray(pinf, np.float64)
    n = in6.shape[0]
    out = np.zeros((n, 3))
    it = np.zeros(n, np.int32)
    dp = C.POINTER(C.c_double)
    sp = seed.ctypes.data_as(dp) if seed is not None else C.cast(None, dp)
    lib().po_mgfm_batched(in6.ctypes.data_as(dp), mat2.ctypes.data_as(C.POINTER(C.c_int8)),
                          gam.ctypes.data_as(dp), pinf.ctypes.data_as(dp), int(variant), sp,
                          out.ctypes.data_as(dp), it.ctypes.data_as(C.POINTER(C.c_int32)), n)
    return out, it


def root_d(x, d):
    return lib().po_root_d(float(x), int(d))

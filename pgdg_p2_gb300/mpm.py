"""Host-side mirror of the reference's MPM method set over libpgdg_gpu.so.

`MPM` wraps one device context and exposes the methods the 3D_generalized
driver calls (3D_generalized/PGDG_3D_spheric/mpm.h:160-194) under the same
names: Set_timestep, Used_state_update, Map_the_particle_to_tree,
Split_particle_fast, Merge_particle_fast, MLS_P2G, Calculate_limiter,
Grid_acceleration, Update_grid, Update_particle and MPM_run_simulation.  Every
call goes through the C ABI in include/pgdg.h; a failing call raises PgdgError
with the library's error text.  There is no CPU fallback: without the CUDA
library or a GPU, construction fails.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from .abi import (PREC_FP64, PREC_MIXED, Cells, Particles, PgdgError,  # noqa: F401
                  check, declare_case_builder, pgdg_case, pgdg_cells, pgdg_particles, pgdg_stats)

_libs = {}


def lib(nfld=2):
    """Load (building first if needed) the in-tree library of a material count:
    libpgdg_gpu.so (two materials) or libpgdg_gpu_f3.so (the three-material build)."""
    if nfld not in _libs:
        path = _build.lib_path(nfld)
        if not os.path.exists(path) or os.environ.get("PGDG_REBUILD"):
            _build.build()
        L = C.CDLL(path)
        P = C.POINTER
        vp = C.c_void_p
        declare_case_builder(L)
        L.pgdg_create.argtypes = [P(pgdg_case), C.c_int, C.c_int64, P(vp)]
        L.pgdg_last_error.argtypes = [vp]
        L.pgdg_last_error.restype = C.c_char_p
        for name in ("pgdg_destroy", "pgdg_used_state_update", "pgdg_bin_particles", "pgdg_split_particle_fast",
                     "pgdg_merge_particle_fast", "pgdg_refresh_membership", "pgdg_refresh_neighbors",
                     "pgdg_mls_p2g", "pgdg_calculate_limiter", "pgdg_grid_acceleration", "pgdg_synchronize"):
            getattr(L, name).argtypes = [vp]
        L.pgdg_capacity.argtypes = [vp, P(C.c_int64)]
        L.pgdg_upload_particles.argtypes = [vp, P(pgdg_particles)]
        L.pgdg_download_particles.argtypes = [vp, P(pgdg_particles)]
        L.pgdg_num_particles.argtypes = [vp, P(C.c_int64)]
        L.pgdg_upload_cells.argtypes = [vp, P(pgdg_cells)]
        L.pgdg_download_cells.argtypes = [vp, P(pgdg_cells)]
        L.pgdg_upload_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64)]
        L.pgdg_download_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64), P(C.c_int32), C.c_int64, P(C.c_int64)]
        L.pgdg_download_cell_lists.argtypes = [vp, P(C.c_int64), P(C.c_int64), C.c_int64, P(C.c_int64)]
        L.pgdg_set_dt.argtypes = [vp, C.c_double]
        L.pgdg_set_iterate.argtypes = [vp, C.c_int64]
        L.pgdg_set_max_v.argtypes = [vp, C.c_double]
        L.pgdg_get_stats.argtypes = [vp, P(pgdg_stats)]
        L.pgdg_set_timestep.argtypes = [vp, P(C.c_double), P(C.c_double)]
        L.pgdg_update_grid.argtypes = [vp, C.c_int]
        L.pgdg_update_particle.argtypes = [vp, C.c_int]
        L.pgdg_run_step.argtypes = [vp, C.c_int64]
        L.pgdg_advance.argtypes = [vp, C.c_int]
        L.pgdg_totals.argtypes = [vp, P(C.c_double)]
        L.pgdg_output_point.argtypes = [vp, P(C.c_double)]
        L.pgdg_case_build.argtypes = [vp, C.c_int, C.c_uint64]
        L.pgdg_output_plt.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int]
        L.pgdg_output_wait.argtypes = [vp]
        L.pgdg_profile.argtypes = [vp, C.c_int]
        L.pgdg_profile_read.argtypes = [vp, C.c_char_p, C.c_int, P(C.c_double), P(C.c_int64), C.c_int, P(C.c_int)]
        L.pgdg_launch_count.argtypes = [vp, P(C.c_int64)]
        L.pgdg_time_advance.argtypes = [vp, C.c_int, P(C.c_double)]
        L.pgdg_fp32_peak.argtypes = [P(C.c_double), P(C.c_double)]
        L.pgdg_fp32_peak_packed.argtypes = [P(C.c_double), P(C.c_double)]
        L.pgdg_mgfm_batched.argtypes = [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp, vp, C.c_int64]
        L.pgdg_mgfm_batched_noalloc.argtypes = [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp, vp, C.c_int64]
        L.pgdg_surrogate_create.argtypes = [C.c_int, P(vp)]
        L.pgdg_surrogate_destroy.argtypes = [vp]
        L.pgdg_surrogate_num_params.restype = C.c_int
        L.pgdg_surrogate_set_params.argtypes = [vp, P(C.c_float)]
        L.pgdg_surrogate_get_params.argtypes = [vp, P(C.c_float)]
        L.pgdg_surrogate_features.argtypes = [vp, vp, vp, vp, vp, C.c_int64]
        L.pgdg_surrogate_forward.argtypes = [vp, vp, vp, C.c_int64]
        L.pgdg_surrogate_gradients.argtypes = [vp, vp, vp, C.c_int64, P(C.c_float), P(C.c_double)]
        L.pgdg_surrogate_train_step.argtypes = [vp, vp, vp, C.c_int64, C.c_float, P(C.c_double)]
        L.pgdg_set_surrogate.argtypes = [vp, vp]
        L.pgdg_set_iface_queue.argtypes = [vp, C.c_int]
        L.pgdg_tune.argtypes = [vp, C.c_char_p, C.c_int, P(C.c_int)]
        L.pgdg_set_graphs.argtypes = [vp, C.c_int]
        L.pgdg_iface_download.argtypes = [vp, vp, vp, C.c_int64, P(C.c_int64)]
        _libs[nfld] = L
    return _libs[nfld]


# ---------------------------------------------------------------------------
# case construction (MPM::Initialize_case restated for the synthetic workloads)
# ---------------------------------------------------------------------------
def case_setup(config_id, ncell=None):
    cs = pgdg_case()
    nc = (C.c_int32 * 3)(*(ncell or (0, 0, 0)))
    check(lib().pgdg_case_setup(int(config_id), nc, C.byref(cs)), "pgdg_case_setup")
    return cs


def case_particles(cs, config_id, seed=0):
    n = lib().pgdg_case_num_particles(C.byref(cs))
    p = Particles(n, cs.dim)
    v = p.view()
    check(lib().pgdg_case_particles(C.byref(cs), int(config_id), int(seed), C.byref(v)), "pgdg_case_particles")
    return p


def case_cells(cs):
    c = Cells(cs.ncells, cs.dim, nfld=cs.nfld)
    check(lib().pgdg_case_cells(C.byref(cs), C.byref(c.view())), "pgdg_case_cells")
    return c


def make_case(config_id, ncell=None, seed=0):
    cs = case_setup(config_id, ncell)
    return cs, case_particles(cs, config_id, seed), case_cells(cs)


class MPM:
    """One device context (one case, one GPU)."""

    def __init__(self, cs: pgdg_case, precision=PREC_FP64, capacity=0):
        self.cs = cs
        self.dim = cs.dim
        self.h = C.c_void_p()
        self._L = lib(cs.nfld)
        rc = self._L.pgdg_create(C.byref(cs), int(precision), int(capacity), C.byref(self.h))
        if rc != 0:
            raise PgdgError(rc, "pgdg_create")

    def close(self):
        if getattr(self, "h", None):
            self._L.pgdg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            msg = self._L.pgdg_last_error(self.h)
            raise PgdgError(rc, f"{what}: {msg.decode() if msg else ''}")

    def sync(self):
        self._ck(self._L.pgdg_synchronize(self.h), "pgdg_synchronize")

    # ---- state exchange ----
    def case_build(self, config_id, seed=0):
        """Build workload config_id (this context's case) in place on the device."""
        self._ck(self._L.pgdg_case_build(self.h, int(config_id), int(seed)), "case_build")

    def upload_particles(self, p: Particles):
        v = p.view()
        v.n = p.n
        self._ck(self._L.pgdg_upload_particles(self.h, C.byref(v)), "upload_particles")

    def num_particles(self):
        n = C.c_int64()
        self._ck(self._L.pgdg_num_particles(self.h, C.byref(n)), "num_particles")
        return n.value

    def download_particles(self, out=None):
        """The live particles in canonical order (into `out` when given: a
        Particles with room for them, e.g. in page-locked memory)."""
        n = self.num_particles()
        p = out if out is not None else Particles(n, self.dim)
        if p.cap < n:
            raise PgdgError(-1, "download_particles: out too small")
        v = p.view()
        self._ck(self._L.pgdg_download_particles(self.h, C.byref(v)), "download_particles")
        p.n = int(v.n)
        return p

    def upload_cells(self, c: Cells):
        self._ck(self._L.pgdg_upload_cells(self.h, C.byref(c.view())), "upload_cells")

    def download_cells(self, out=None):
        c = out if out is not None else Cells(self.cs.ncells, self.dim, nfld=self.cs.nfld)
        self._ck(self._L.pgdg_download_cells(self.h, C.byref(c.view())), "download_cells")
        return c

    def upload_lists(self, off, ent):
        off = np.ascontiguousarray(off, np.int64)
        ent = np.ascontiguousarray(ent if len(ent) else np.zeros(1, np.int64), np.int64)
        self._ck(self._L.pgdg_upload_lists(self.h, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                         ent.ctypes.data_as(C.POINTER(C.c_int64))), "upload_lists")

    def download_lists(self):
        n = self.num_particles()
        tot = C.c_int64()
        off = np.zeros(n + 1, np.int64)
        stored = np.zeros(max(n, 1), np.int32)
        P = C.POINTER
        self._ck(self._L.pgdg_download_lists(self.h, off.ctypes.data_as(P(C.c_int64)), None,
                                           stored.ctypes.data_as(P(C.c_int32)), 0, C.byref(tot)), "download_lists")
        ent = np.zeros(max(tot.value, 1), np.int64)
        self._ck(self._L.pgdg_download_lists(self.h, off.ctypes.data_as(P(C.c_int64)), ent.ctypes.data_as(P(C.c_int64)),
                                           stored.ctypes.data_as(P(C.c_int32)), ent.size, C.byref(tot)),
                 "download_lists")
        return off, ent[: tot.value], stored[:n]

    def download_cell_lists(self):
        tot = C.c_int64()
        off = np.zeros(self.cs.ncells + 1, np.int64)
        P = C.POINTER
        self._ck(self._L.pgdg_download_cell_lists(self.h, off.ctypes.data_as(P(C.c_int64)), None, 0, C.byref(tot)),
                 "download_cell_lists")
        ent = np.zeros(max(tot.value, 1), np.int64)
        self._ck(self._L.pgdg_download_cell_lists(self.h, off.ctypes.data_as(P(C.c_int64)),
                                                ent.ctypes.data_as(P(C.c_int64)), ent.size, C.byref(tot)),
                 "download_cell_lists")
        return off, ent[: tot.value]

    def set_dt(self, dt):
        self._ck(self._L.pgdg_set_dt(self.h, float(dt)), "set_dt")

    def set_iterate(self, n):
        self._L.pgdg_set_iterate(self.h, int(n))

    def set_max_v(self, mv):
        self._ck(self._L.pgdg_set_max_v(self.h, float(mv)), "set_max_v")

    def set_surrogate(self, net):
        """Seed every interface MGFM solve of the mixed step with `net` (None: plain)."""
        self._ck(self._L.pgdg_set_surrogate(self.h, net.h if net is not None else None), "set_surrogate")

    def tune(self, kernel="pst", variant=-2):
        """Force (variant >= 0), re-tune (-1) or query (-2) a kernel's variant;
        returns the current choice (-1: not tuned yet)."""
        ch = C.c_int()
        self._ck(self._L.pgdg_tune(self.h, kernel.encode(), int(variant), C.byref(ch)), "tune")
        return ch.value

    def set_graphs(self, on):
        """Replay captured CUDA graphs of whole steps in advance() (default on)."""
        self._ck(self._L.pgdg_set_graphs(self.h, 1 if on else 0), "set_graphs")

    def set_iface_queue(self, on):
        """Solve each stage's interface problems as one batch (mixed / FP64_FMA paths)."""
        self._ck(self._L.pgdg_set_iface_queue(self.h, 1 if on else 0), "set_iface_queue")

    def iface_problems(self):
        """The last stage's queued interface problems: (in6 [n,6], mat2 [n,2])."""
        n = C.c_int64()
        z6, z2 = np.zeros((1, 6)), np.zeros((1, 2), np.int8)
        self._ck(self._L.pgdg_iface_download(self.h, z6.ctypes.data, z2.ctypes.data, 0, C.byref(n)), "iface_download")
        in6, mat = np.zeros((max(n.value, 1), 6)), np.zeros((max(n.value, 1), 2), np.int8)
        self._ck(self._L.pgdg_iface_download(self.h, in6.ctypes.data, mat.ctypes.data, n.value, C.byref(n)),
                 "iface_download")
        return in6[:n.value], mat[:n.value]

    def stats(self):
        s = pgdg_stats()
        self._ck(self._L.pgdg_get_stats(self.h, C.byref(s)), "stats")
        return s.to_dict()

    def output_point(self):
        """Output_point's bubble probe: (downstream end, jet, upstream end, phase-2 mass, fluid count)."""
        out = np.zeros(5)
        self._ck(self._L.pgdg_output_point(self.h, out.ctypes.data_as(C.POINTER(C.c_double))), "output_point")
        return out

    def output_plt(self, particle_path=None, cell_path=None, async_write=False):
        """Output_plt_file: the particle Tecplot binary and the cell table.  With
        async_write the call returns once the snapshot is packed on the device;
        output_wait() joins the writer."""
        enc = (lambda p: str(p).encode() if p is not None else None)
        self._ck(self._L.pgdg_output_plt(self.h, enc(particle_path), enc(cell_path), 1 if async_write else 0),
                 "output_plt")

    def output_wait(self):
        self._ck(self._L.pgdg_output_wait(self.h), "output_wait")

    def totals(self):
        """Particle mass per phase, particle energy, cell mass per phase, cell energy."""
        out = np.zeros(2 * self.cs.nfld + 2)
        self._ck(self._L.pgdg_totals(self.h, out.ctypes.data_as(C.POINTER(C.c_double))), "totals")
        return out

    # ---- reference methods ----
    def Set_timestep(self):
        dt, mv = C.c_double(), C.c_double()
        self._ck(self._L.pgdg_set_timestep(self.h, C.byref(dt), C.byref(mv)), "Set_timestep")
        return dt.value, mv.value

    def Used_state_update(self):
        self._ck(self._L.pgdg_used_state_update(self.h), "Used_state_update")

    def Map_the_particle_to_tree(self):
        self._ck(self._L.pgdg_bin_particles(self.h), "Map_the_particle_to_tree")

    def Split_particle_fast(self):
        self._ck(self._L.pgdg_split_particle_fast(self.h), "Split_particle_fast")

    def Merge_particle_fast(self):
        self._ck(self._L.pgdg_merge_particle_fast(self.h), "Merge_particle_fast")

    def Refresh_membership(self):
        self._ck(self._L.pgdg_refresh_membership(self.h), "Refresh_membership")

    def Refresh_neighbors(self):
        self._ck(self._L.pgdg_refresh_neighbors(self.h), "Refresh_neighbors")

    def MLS_P2G(self):
        self._ck(self._L.pgdg_mls_p2g(self.h), "MLS_P2G")

    def Calculate_limiter(self):
        self._ck(self._L.pgdg_calculate_limiter(self.h), "Calculate_limiter")

    def Grid_acceleration(self):
        self._ck(self._L.pgdg_grid_acceleration(self.h), "Grid_acceleration")

    def Update_grid(self, md):
        self._ck(self._L.pgdg_update_grid(self.h, int(md)), "Update_grid")

    def Update_particle(self, md):
        self._ck(self._L.pgdg_update_particle(self.h, int(md)), "Update_particle")

    def MPM_run_simulation(self, n):
        self._ck(self._L.pgdg_run_step(self.h, int(n)), "MPM_run_simulation")

    def advance(self, nsteps):
        self._ck(self._L.pgdg_advance(self.h, int(nsteps)), "advance")

    # ---- measurement ----
    def time_advance(self, nsteps):
        """Device time (ms) of nsteps steps, CUDA events on the context stream."""
        ms = C.c_double()
        self._ck(self._L.pgdg_time_advance(self.h, int(nsteps), C.byref(ms)), "time_advance")
        return ms.value

    def profile(self, enable=True):
        self._ck(self._L.pgdg_profile(self.h, 1 if enable else 0), "profile")

    def profile_read(self):
        names = C.create_string_buffer(4096)
        ms = (C.c_double * 64)()
        cnt = (C.c_int64 * 64)()
        n = C.c_int()
        self._ck(self._L.pgdg_profile_read(self.h, names, 4096, ms, cnt, 64, C.byref(n)), "profile_read")
        keys = names.value.decode().split(";")[: n.value]
        return {k: (ms[i], cnt[i]) for i, k in enumerate(keys)}

    def launch_count(self):
        n = C.c_int64()
        self._ck(self._L.pgdg_launch_count(self.h, C.byref(n)), "launch_count")
        return n.value


def fp32_peak(packed=False):
    """Measured FP32 multiply-add rate of the current device (packed: FFMA2
    pairs): (TFLOP/s, ms of the timed launch)."""
    tf, ms = C.c_double(), C.c_double()
    fn = lib().pgdg_fp32_peak_packed if packed else lib().pgdg_fp32_peak
    check(fn(C.byref(tf), C.byref(ms)), "pgdg_fp32_peak")
    return tf.value, ms.value

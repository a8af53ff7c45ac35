"""ctypes mirror of include/pgdg_types.h (data formats only) and numpy helpers.

The structures are the plain-C layouts of the library boundary; `Particles` and
`Cells` hold numpy arrays and hand out `pgdg_particles` / `pgdg_cells` views of
them.  Field meanings follow the reference's Particle_base / MPM members
(3D_generalized/PGDG_3D_spheric/particle.h:9-106, mpm.h:52-195).
"""
import ctypes as C

import numpy as np

PGDG_OK = 0
ERRORS = {
    -1: "PGDG_EINVAL", -2: "PGDG_ENOMEM", -3: "PGDG_ECUDA", -4: "PGDG_ENONFINITE",
    -5: "PGDG_ETIMEOUT", -6: "PGDG_EOVERFLOW", -7: "PGDG_ESTATE",
}
BC_INTERIOR, BC_WALL, BC_INLET, BC_OUTLET, BC_SYMMETRY, BC_TRANSMISSIVE = 0, 1, -1, -2, -3, -4
MGFM_3D, MGFM_2D = 0, 1
PREC_FP64, PREC_MIXED, PREC_FP64_FMA = 0, 1, 2
F = 2            # materials of the default build
MAX_FLD = 3      # PGDG_MAX_FLD: the largest material count of a build


class PgdgError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__(f"{what}: {ERRORS.get(code, code)}")
        self.code = code


def check(code, what=""):
    if code != PGDG_OK:
        raise PgdgError(code, what)


class pgdg_case(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("nfld", C.c_int32), ("ncell", C.c_int32 * 3), ("bc", C.c_int32 * 6),
        ("mgfm_variant", C.c_int32), ("merge_iters", C.c_int32),
        ("box_l", C.c_double * 3), ("box_r", C.c_double * 3), ("p_size", C.c_double * 3),
        ("p_g", C.c_double), ("p_sz", C.c_double),
        ("gamma", C.c_double * MAX_FLD), ("pinf", C.c_double * MAX_FLD), ("ini_rho", C.c_double * MAX_FLD),
        ("c_ini", C.c_double * MAX_FLD), ("inlet_rho", C.c_double), ("inlet_u", C.c_double * 3),
        ("inlet_p", C.c_double), ("cfl", C.c_double), ("probe", (C.c_double * 3) * 8),
    ]

    @property
    def ncells(self):
        return self.ncell[0] * self.ncell[1] * (self.ncell[2] if self.dim == 3 else 1)

    def to_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if name == "probe":
                out[name] = [list(r) for r in v]
            elif hasattr(v, "__len__"):
                out[name] = list(v)
            else:
                out[name] = v
        return out

    @classmethod
    def from_dict(cls, d):
        cs = cls()
        for name, _ in cls._fields_:
            v = d[name]
            if name == "probe":
                for i in range(8):
                    for j in range(3):
                        cs.probe[i][j] = v[i][j]
            elif isinstance(v, list):
                arr = getattr(cs, name)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(cs, name, v)
        return cs


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint64)


class pgdg_particles(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("coord", _dp), ("v", _dp), ("tv", _dp), ("rhov", _dp),
        ("vol", _dp), ("mass", _dp), ("h", _dp), ("P", _dp), ("rho", _dp), ("E", _dp), ("c", _dp),
        ("slope", _dp), ("phase", _ip), ("mark_in", _ip), ("seq", _up),
    ]


class pgdg_cells(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("rho", _dp), ("rhov", _dp), ("E", _dp), ("c", _dp), ("ac", _dp),
        ("alph", _dp), ("coef", _dp), ("v", _dp), ("P", _dp), ("ph_state", _ip),
        ("ph_state_b", _ip), ("used", _ip), ("lim_u", _dp), ("g_v", _dp), ("dcoef", _dp),
    ]


class pgdg_stats(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64), ("n_split", C.c_int64), ("n_inlet", C.c_int64),
        ("n_outlet", C.c_int64), ("n_merge", C.c_int64), ("n_affected", C.c_int64),
        ("mgfm_calls", C.c_int64), ("mgfm_iters", C.c_int64), ("mgfm_maxit_hits", C.c_int64),
        ("g2p_fallbacks", C.c_int64), ("list_entries", C.c_int64), ("iterate_num", C.c_int64),
        ("dt", C.c_double), ("max_v", C.c_double), ("time", C.c_double),
    ]

    def to_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


PARTICLE_FIELDS = {
    # name: (components per particle or callable(dim), dtype)
    "coord": 3, "v": 3, "tv": 3, "rhov": 3, "vol": 1, "mass": 1, "h": 1, "P": 1, "rho": 1,
    "E": 1, "c": 1, "slope": None, "phase": 1, "mark_in": 1, "seq": 1,
}


class Particles:
    """numpy arrays of fluid particles (canonical order).  alloc(shape, dtype)
    may supply the arrays (e.g. page-locked host memory); default np.zeros."""

    def __init__(self, n, dim, alloc=None):
        z = alloc or np.zeros
        self.dim = dim
        self.cap = int(n)
        self.n = int(n)
        U = dim + 2
        ns = U * dim
        f8 = np.float64
        self.coord = z((n, 3), f8)
        self.v = z((n, 3), f8)
        self.tv = z((n, 3), f8)
        self.rhov = z((n, 3), f8)
        for k in ("vol", "mass", "h", "P", "rho", "E", "c"):
            setattr(self, k, z((n,), f8))
        self.slope = z((n, ns), f8)
        self.phase = z((n,), np.int32)
        self.mark_in = z((n,), np.int32)
        self.seq = z((n,), np.uint64)

    NAMES = ("coord", "v", "tv", "rhov", "vol", "mass", "h", "P", "rho", "E", "c", "slope",
             "phase", "mark_in", "seq")

    def view(self):
        s = pgdg_particles()
        s.n = self.cap
        for k in self.NAMES:
            a = getattr(self, k)
            ct = C.c_double if a.dtype == np.float64 else (C.c_int32 if a.dtype == np.int32 else C.c_uint64)
            setattr(s, k, _ptr(a, ct))
        return s

    def trim(self, n):
        self.n = int(n)
        for k in self.NAMES:
            setattr(self, k, getattr(self, k)[: self.n].copy())
        self.cap = self.n
        return self

    def copy(self):
        o = Particles(self.n, self.dim)
        for k in self.NAMES:
            setattr(o, k, getattr(self, k).copy())
        return o

    def as_dict(self):
        return {k: getattr(self, k) for k in self.NAMES}


class Cells:
    """numpy SoA of grid cells (lexicographic (i*NY+j)*NZ+k)."""

    NAMES = ("rho", "rhov", "E", "c", "ac", "alph", "coef", "v", "P", "ph_state", "ph_state_b",
             "used", "lim_u", "g_v", "dcoef")

    def __init__(self, n, dim, alloc=None, nfld=F):
        z = alloc or np.zeros
        self.dim = dim
        self.n = int(n)
        self.nfld = nf = int(nfld)
        U, B = dim + 2, dim + 1
        f8 = np.float64
        self.rho = z((n, nf), f8)
        self.rhov = z((n, nf, 3), f8)
        self.E = z((n, nf), f8)
        self.c = z((n, nf), f8)
        self.ac = z((n, nf), f8)
        self.alph = z((n, nf), f8)
        self.coef = z((n, nf, U, B), f8)
        self.v = z((n, 3), f8)
        self.P = z((n,), f8)
        self.ph_state = z((n, nf), np.int32)
        self.ph_state_b = z((n, nf), np.int32)
        self.used = z((n,), np.int32)
        self.lim_u = z((n, nf, U), f8)
        self.g_v = z((n, dim, dim), f8)
        self.dcoef = z((n, nf, U, B), f8)

    def view(self):
        s = pgdg_cells()
        s.n = self.n
        for k in self.NAMES:
            a = getattr(self, k)
            ct = C.c_double if a.dtype == np.float64 else C.c_int32
            setattr(s, k, _ptr(a, ct))
        return s

    def copy(self):
        o = Cells(self.n, self.dim, nfld=self.nfld)
        for k in self.NAMES:
            setattr(o, k, getattr(self, k).copy())
        return o

    def as_dict(self):
        return {k: getattr(self, k) for k in self.NAMES}


def declare_case_builder(lib):
    lib.pgdg_case_setup.argtypes = [C.c_int, C.POINTER(C.c_int32), C.POINTER(pgdg_case)]
    lib.pgdg_case_num_particles.argtypes = [C.POINTER(pgdg_case)]
    lib.pgdg_case_num_particles.restype = C.c_int64
    lib.pgdg_case_particles.argtypes = [C.POINTER(pgdg_case), C.c_int, C.c_uint64, C.POINTER(pgdg_particles)]
    lib.pgdg_case_cells.argtypes = [C.POINTER(pgdg_case), C.POINTER(pgdg_cells)]

"""Host-side case construction (MPM::Initialize_case restated for the workloads)."""
import math

import numpy as np
import pytest

from pgdg_p2_gb300 import mpm as M
from pgdg_p2_gb300.abi import BC_INLET, BC_OUTLET, BC_SYMMETRY, BC_TRANSMISSIVE, BC_WALL


def test_post_shock_state():
    cs = M.case_setup(3)
    # Rankine-Hugoniot for a Mach 1.22 shock into air at rest (gamma 1.4, rho 1, p 1)
    assert cs.inlet_p == pytest.approx(1.5698, abs=1e-4)
    assert cs.inlet_rho == pytest.approx(1.3764, abs=1e-4)
    assert cs.inlet_u[0] == pytest.approx(0.3947, abs=1e-4)


@pytest.mark.parametrize("cid,grid,ppc,n", [(1, (112, 48), 4, 21504), (2, (256, 64, 64), 8, 8388608),
                                            (3, (384, 96, 96), 8, 28311552), (4, (1024, 1024), 4, 4194304)])
def test_sizes(cid, grid, ppc, n):
    cs = M.case_setup(cid)
    assert list(cs.ncell[:cs.dim]) == list(grid)
    assert M.lib().pgdg_case_num_particles(M.C.byref(cs)) == n
    assert cs.ncells * ppc == n
    assert cs.p_sz == pytest.approx(cs.p_g / 2, rel=1e-12)


def test_boundary_kinds():
    assert list(M.case_setup(3).bc) == [BC_INLET, BC_OUTLET, BC_SYMMETRY, BC_WALL, BC_SYMMETRY, BC_WALL]
    assert list(M.case_setup(2).bc) == [BC_INLET, BC_OUTLET, BC_SYMMETRY, BC_WALL, BC_SYMMETRY, BC_SYMMETRY]
    assert list(M.case_setup(1).bc)[:4] == [BC_WALL] * 4
    assert list(M.case_setup(4).bc)[:4] == [BC_TRANSMISSIVE] * 4


def test_regions_sphere():
    cs, p, c = M.make_case(3, (48, 12, 12))
    x = p.coord
    inside = (x[:, 0] - 1.5) ** 2 + x[:, 1] ** 2 + x[:, 2] ** 2 < 0.0625
    assert np.all(p.phase[inside] == 2) and np.all(p.phase[~inside] == 1)
    assert np.allclose(p.rho[inside], 0.138)
    shocked = x[:, 0] < 1.0
    assert np.allclose(p.rhov[shocked, 0] / p.rho[shocked], cs.inlet_u[0])
    assert np.all(p.vol == cs.p_sz * cs.p_sz * cs.p_sz)
    assert np.array_equal(p.seq, np.arange(p.n, dtype=np.uint64))


def test_jitter_triple_point():
    cs, p, c = M.make_case(1)
    # 2x2 sub-lattice at +-dx/4 with seeded uniform jitter in +-dx/8
    cell = np.floor(p.coord[:, :2] / cs.p_g)
    off = p.coord[:, :2] - (cell + 0.5) * cs.p_g
    assert np.all(np.abs(np.abs(off) - cs.p_g / 4) <= cs.p_g / 8 + 1e-15)
    cs2, p2, _ = M.make_case(1)
    assert np.array_equal(p.coord, p2.coord)
    top = (p.coord[:, 0] > 1) & (p.coord[:, 1] > 1.5)
    assert np.all(p.phase[top] == 2) and np.allclose(p.rho[top], 0.125)


def test_undex_stiffened_gas():
    cs, p, c = M.make_case(4, (64, 64))
    water = p.phase == 1
    assert cs.pinf[0] == 3.309e8 and cs.gamma[0] == 7.15
    assert np.allclose(p.c[water], math.sqrt(7.15 * (1e5 + 3.309e8) / 1000))


@pytest.mark.parametrize("cid,grid,seed", [(1, None, 0), (1, (56, 24), 77), (2, (32, 8, 8), 0), (3, (48, 12, 12), 0),
                                           (3, (96, 24, 24), 0), (4, (64, 64), 0), (2, None, 0), (3, None, 0),
                                           (4, None, 0), (5, None, 0), (5, (56, 24), 9)])
def test_oracle_case_builder_bitwise(cid, grid, seed):
    """The oracle's own case construction (used by the CPU arms of the bench,
    which load no GPU library) equals the library's bit for bit: the case
    parameters always, particles and cells where the case fits a CPU test."""
    from oracle import oracle as O
    cs_g, cs_o = M.case_setup(cid, grid), O.case_setup(cid, grid)
    assert bytes(cs_g) == bytes(cs_o)
    if grid is None and cid != 1:
        return
    pg, po = M.case_particles(cs_g, cid, seed), O.case_particles(cs_o, cid, seed)
    assert pg.n == po.n
    for k in pg.NAMES:
        assert getattr(pg, k).tobytes() == getattr(po, k).tobytes(), k
    cg, co = M.case_cells(cs_g), O.case_cells(cs_o)
    for k in ("rho", "rhov", "E", "c", "ac", "alph", "coef", "v", "P", "ph_state", "ph_state_b", "used", "lim_u",
              "g_v", "dcoef"):
        assert getattr(cg, k).tobytes() == getattr(co, k).tobytes(), k


def test_three_material_regions():
    """Triple_point_3phase (mpm_ini.cpp:80-97, 157-245): lower right phase 1,
    upper right phase 2, left phase 3 (stiffened, p_inf 0.1), on C1's box."""
    cs, p, c = M.make_case(5)
    assert cs.nfld == 3 and cs.dim == 2 and tuple(cs.ncell[:2]) == (112, 48)
    assert list(cs.gamma) == [1.4, 1.5, 1.6] and list(cs.pinf) == [0, 0, 0.1]
    x, y = p.coord[:, 0], p.coord[:, 1]
    assert np.all(p.phase[(x > 1) & (y < 1.5)] == 1)
    assert np.all(p.phase[(x > 1) & (y >= 1.5)] == 2)
    assert np.all(p.phase[x <= 1] == 3)
    left = p.phase == 3
    assert np.allclose(p.P[left], 1.0) and np.allclose(p.E[left], (1.0 + 1.6 * 0.1) / 0.6)
    assert c.rho.shape == (cs.ncells, 3)

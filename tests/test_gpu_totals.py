"""Conservation totals (Triple_point_2phase/mpm_ini.cpp:599-654: particle mass
per phase, particle energy, cell mass per phase, cell energy) and the bubble
probe (Output_point, mpm_ini.cpp:774-824) against the oracle's.  Totals sum in
double-double and round once on both sides, so the exact-order FP64 path,
whose addends equal the oracle's bit for bit, gives the same six doubles.

The mixed path's totals are sums of the conserved cell and particle fields
whose relative L1 error the accuracy gate bounds by 1e-3, and
|sum (q - q_ref)| <= sum |q - q_ref|, so 1e-3 bounds them too; the test holds
them to MIXED_TOL = 1e-4, or 3x the oracle's own change under FP32-sized
perturbation of its input where that is larger.  Particle mass is re-derived
every stage as vol * rho from the cell polynomial (Update_state_onestep,
particle_flow.cpp:413-477) and falls back to the cell average where the
reconstructed pressure fails the positivity test, a discrete switch that
FP32 rounding moves: the underwater explosion's gas mass shows 3e-5 after
five steps."""
import numpy as np
import pytest

from tests.golden.make_golden import CASES
from tests.gpu_helpers import fp32_perturbed

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-4


@pytest.mark.parametrize("name,cid,grid,steps", CASES)
def test_totals_vs_oracle(gpu_mod, oracle_mod, name, cid, grid, steps):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64, PREC_MIXED
    cs, p, c = M.make_case(cid, grid[:2] if grid[2] == 1 else grid)
    o, ob = O.Oracle(cs), O.Oracle(cs)
    ctx = {"exact": M.MPM(cs, PREC_FP64), "mixed": M.MPM(cs, PREC_MIXED)}
    for x in (o, *ctx.values()):
        x.upload_particles(p)
    ob.upload_particles(fp32_perturbed(p))
    for x in (o, ob, *ctx.values()):
        x.upload_cells(c)
    for s in range(1, steps + 1):
        dt, mv = o.Set_timestep()
        for g in (ob, *ctx.values()):
            g.Set_timestep()
            g.set_dt(dt)
            g.set_max_v(mv)
        for x in (o, ob, *ctx.values()):
            x.set_iterate(s)
            x.MPM_run_simulation(s)
    to = o.totals()
    assert np.all(np.isfinite(to)) and to[0] > 0 and to[3] > 0
    te = ctx["exact"].totals()
    assert te.tobytes() == to.tobytes(), (te, to)
    tm, tb = ctx["mixed"].totals(), ob.totals()
    scale = np.maximum(np.abs(to), 1e-300)
    rel, floor = np.abs(tm - to) / scale, np.abs(tb - to) / scale
    print(name, "mixed rel", rel, "floor", floor, "fallbacks", ctx["mixed"].stats()["g2p_fallbacks"],
          o.stats()["g2p_fallbacks"])
    assert np.all(rel <= np.maximum(MIXED_TOL, 3 * floor)), (rel, floor)


@pytest.mark.parametrize("cid,grid,steps", [(3, (48, 12, 12), 6), (2, (32, 8, 8), 4), (1, (112, 48), 20)])
def test_output_point_vs_oracle(gpu_mod, oracle_mod, cid, grid, steps):
    """MPM::Output_point: the bubble's axial extents, the phase-2 mass and the
    particle count; the exact path equals the oracle bit for bit (min/max,
    and the mass summed in double-double)."""
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, p, c = M.make_case(cid, grid)
    g, o = M.MPM(cs, PREC_FP64), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(p)
        x.upload_cells(c)
        x.advance(steps)
    pg, po = g.output_point(), o.output_point()
    assert pg.tobytes() == po.tobytes(), (pg, po)
    assert po[4] == o.num_particles() and po[3] > 0
    if cs.dim == 3:
        # the sphere's axial ends near t = 0: x = 1.5 -+ 0.25 within two particle spacings
        assert abs(po[0] - 1.75) < 2 * cs.p_sz and abs(po[1] - 1.25) < 2 * cs.p_sz

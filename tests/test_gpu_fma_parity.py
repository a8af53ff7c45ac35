"""The plain FP64 GPU path (PGDG_PREC_FP64_FMA: FP64 with FMA contraction,
row-sorted shifting sums, the path the mixed one is measured against) against
the FP64 oracle, kernel by kernel on identical inputs: relative error
sum |a - b| / sum |b| <= 1e-12 per output field.

Each method starts from the same oracle state (the golden cases after their
golden step counts); cell methods get the oracle's cells re-uploaded before
the call, so every comparison is of one call on identical FP64 inputs.  The
limiter is compared through the limited slopes Lim_u * slope it hands the
residual: where a slope is nearly zero its limiter is a ratio of rounding
noise (Calculate_limiter, mpm.cpp:392-738) and any change of rounding moves
it, while the product stays at rounding level."""
import numpy as np
import pytest

from tests.golden.make_golden import CASES

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rel(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


@pytest.mark.parametrize("name,cid,grid,steps", CASES)
def test_fp64_fma_methods_vs_oracle(gpu_mod, oracle_mod, name, cid, grid, steps):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64_FMA
    cs, p, c = M.make_case(cid, grid[:2] if grid[2] == 1 else grid)
    o0 = O.Oracle(cs)
    o0.upload_particles(p)
    o0.upload_cells(c)
    o0.advance(steps)
    ps, cst = o0.download_particles(), o0.download_cells()
    off, ent = o0.download_lists()
    st = o0.stats()
    g, o = M.MPM(cs, PREC_FP64_FMA), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(ps)
        x.upload_cells(cst)
        x.upload_lists(off, ent)
        x.set_iterate(steps + 1)
        x.set_dt(st["dt"])
        x.set_max_v(st["max_v"])
    F, U, B = 2, cs.dim + 2, cs.dim + 1
    errs = {}
    for x in (g, o):
        x.Map_the_particle_to_tree()
        x.Split_particle_fast()
        for _ in range(cs.merge_iters):
            x.Merge_particle_fast()
        x.Refresh_membership()
        x.Refresh_neighbors()
        x.MLS_P2G()
    cg, co = g.download_cells(), o.download_cells()
    errs["p2g alph"], errs["p2g coef"] = _rel(cg.alph, co.alph), _rel(cg.coef, co.coef)
    g.upload_cells(co)
    for x in (g, o):
        x.Calculate_limiter()
    cg, co = g.download_cells(), o.download_cells()
    sl_g = cg.lim_u.reshape(-1, F, U, 1) * cg.coef.reshape(-1, F, U, B)[..., 1:]
    sl_o = co.lim_u.reshape(-1, F, U, 1) * co.coef.reshape(-1, F, U, B)[..., 1:]
    errs["limited slopes"], errs["G_v"] = _rel(sl_g, sl_o), _rel(cg.g_v, co.g_v)
    g.upload_cells(co)
    for x in (g, o):
        x.Grid_acceleration()
    g.sync()
    cg, co = g.download_cells(), o.download_cells()
    errs["dcoef"] = _rel(cg.dcoef, co.dcoef)
    g.upload_cells(co)
    for md in (0, 1):
        for x in (g, o):
            x.Update_grid(md)
        cg, co = g.download_cells(), o.download_cells()
        errs[f"update {md} coef"] = _rel(cg.coef, co.coef)
        g.upload_cells(co)
    for x in (g, o):
        x.Update_particle(0)
    g.sync()
    pg, po = g.download_particles(), o.download_particles()
    assert pg.n == po.n and np.array_equal(pg.seq, po.seq)
    d = cs.dim
    for k in ("vol", "rho", "E", "P", "c", "mass", "h"):
        errs[f"g2p {k}"] = _rel(getattr(pg, k), getattr(po, k))
    errs["g2p coord"] = _rel(pg.coord[:, :d], po.coord[:, :d])
    errs["shift tv - v"] = _rel((pg.tv - pg.v)[:, :d], (po.tv - po.v)[:, :d])
    print(name, {k: f"{v:.1e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if not v <= TOL}
    assert not bad, bad

"""GPU path vs the CPU oracle on the same inputs.

The exact-order FP64 device path (PGDG_PREC_FP64) evaluates every operation in
the oracle's order without FMA contraction, so whole steps -- binning, split,
four merge passes, P2G, limiter, DG residual with MGFM, update, G2P and
shifting -- must agree bit for bit."""
import json
import os

import numpy as np
import pytest

from tests.gpu_helpers import cells_bitwise_equal, particles_bitwise_equal
from tests.golden.make_golden import CASES, digest_cells, digest_particles

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))


@pytest.mark.parametrize("name,cid,grid,steps", CASES)
def test_fp64_steps_bitwise(gpu_mod, oracle_mod, name, cid, grid, steps):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64, pgdg_case
    cs = pgdg_case.from_dict(GOLD[name]["case"])
    p = M.case_particles(cs, cid)
    c = M.case_cells(cs)
    g = M.MPM(cs, PREC_FP64)
    g.upload_particles(p)
    g.upload_cells(c)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    for s in range(steps):
        g.advance(1)
        o.advance(1)
        g.sync()
        pg, po = g.download_particles(), o.download_particles()
        assert particles_bitwise_equal(pg, po) == [], f"step {s + 1}"
    assert cells_bitwise_equal(g.download_cells(), o.download_cells()) == []
    # and the committed digests (pins x86 and Arm runs to the same bits)
    assert digest_particles(g.download_particles(), cs.dim) == GOLD[name]["particles"]
    assert digest_cells(g.download_cells()) == GOLD[name]["cells"]
    sg, so = g.stats(), o.stats()
    for k in ("n_split", "n_merge", "n_inlet", "n_outlet", "mgfm_calls", "mgfm_iters"):
        assert sg[k] == so[k], k


def test_fp64_methods_bitwise_c3(gpu_mod, oracle_mod):
    """Method by method within steps of the 3D case (localises any divergence)."""
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, p, c = M.make_case(3, (32, 8, 8))
    g = M.MPM(cs, PREC_FP64)
    o = O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(p)
        x.upload_cells(c)
    for step in range(1, 4):
        dg, do = g.Set_timestep(), o.Set_timestep()
        assert dg == do
        g.set_iterate(step)
        o.set_iterate(step)
        if step == 1:
            g.Used_state_update()
            o.Used_state_update()
        g.Map_the_particle_to_tree()
        o.Map_the_particle_to_tree()
        assert [np.array_equal(a, b) for a, b in zip(g.download_cell_lists(), o.download_cell_lists())] == [True, True]
        g.Split_particle_fast()
        o.Split_particle_fast()
        for _ in range(4):
            g.Merge_particle_fast()
            o.Merge_particle_fast()
        o.Refresh_membership()
        for md in range(2):
            o.Refresh_neighbors()
            if md == 0:
                g.MLS_P2G()
                o.MLS_P2G()
                assert cells_bitwise_equal(g.download_cells(), o.download_cells()) == [], "P2G"
            g.Calculate_limiter()
            o.Calculate_limiter()
            assert cells_bitwise_equal(g.download_cells(), o.download_cells(), ("lim_u", "g_v")) == [], "limiter"
            g.Grid_acceleration()
            o.Grid_acceleration()
            assert cells_bitwise_equal(g.download_cells(), o.download_cells(), ("dcoef",)) == [], "residual"
            g.Update_grid(md)
            o.Update_grid(md)
            assert cells_bitwise_equal(g.download_cells(), o.download_cells()) == [], "update"
            g.Update_particle(md)
            o.Update_particle(md)
            assert particles_bitwise_equal(g.download_particles(), o.download_particles()) == [], "G2P/shift"


def test_reupload_restarts_exactly(gpu_mod):
    """Uploading a state into a context that has run steps, with the iteration
    count restarted, continues bit for bit like a fresh context; without the
    restart the cell-based CFL step of the (zero sound-speed) initial cells is
    reported as PGDG_ENONFINITE instead of being used."""
    from pgdg_p2_gb300.abi import PREC_FP64, PgdgError
    M = gpu_mod
    cs, p, c = M.make_case(3, (48, 12, 12))
    fresh = M.MPM(cs, PREC_FP64)
    fresh.upload_particles(p)
    fresh.upload_cells(c)
    fresh.advance(2)
    g = M.MPM(cs, PREC_FP64)
    g.upload_particles(p)
    g.upload_cells(c)
    g.advance(3)
    g.upload_particles(p)
    g.upload_cells(c)
    g.set_iterate(0)
    g.advance(2)
    g.sync()
    assert particles_bitwise_equal(g.download_particles(), fresh.download_particles()) == []
    assert cells_bitwise_equal(g.download_cells(), fresh.download_cells()) == []
    g.upload_particles(p)
    g.upload_cells(c)
    g.set_iterate(5)
    g.advance(1)
    with pytest.raises(PgdgError) as ei:
        g.sync()
    assert ei.value.code == -4   # PGDG_ENONFINITE

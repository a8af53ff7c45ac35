"""Split_particle_fast / Merge_particle_fast on the device: bit-exact per call
against the oracle on identical inputs (particles, cells, neighbour lists),
including the cell-list order and the neighbour lists the passes rebuild."""
import numpy as np
import pytest

from tests.gpu_helpers import particles_bitwise_equal

pytestmark = pytest.mark.gpu


def _lists_match(g, o):
    gof, gent, gst = g.download_lists()
    oof, oent = o.download_lists()
    bad = 0
    for i in np.nonzero(gst)[0]:
        a = gent[gof[i]:gof[i + 1]]
        b = oent[oof[i]:oof[i + 1]]
        b = b[b >= -1]                      # the device keeps no boundary-particle entries
        if not np.array_equal(a, b):
            bad += 1
    return bad


def _event_state(M, O, cid, grid, steps, seed, frac=0.02, outlet=0, inlet=0):
    cs, p, c = M.make_case(cid, grid)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    o.advance(steps)
    po, co = o.download_particles(), o.download_cells()
    off, ent = o.download_lists()
    rng = np.random.default_rng(seed)
    n = po.n
    vmax = cs.p_sz ** cs.dim * 1.6
    vmin = cs.p_sz ** cs.dim * 2 / 3
    idx = rng.choice(n, int(n * frac), replace=False)
    h = len(idx) // 2
    po.vol[idx[:h]] = vmax * rng.uniform(1.01, 2.0, h)              # split candidates
    po.vol[idx[h:]] = vmin * rng.uniform(0.2, 0.99, len(idx) - h)   # merge candidates
    if outlet:
        far = np.argsort(po.coord[:, 0])[-outlet:]
        po.coord[far, 0] = cs.box_r[0] + 1e-3 * cs.p_sz              # leave through the outlet
    if inlet:
        near = np.argsort(po.coord[:, 0])[:inlet]
        po.mark_in[near] = 1
        po.coord[near, 0] = cs.box_l[0] + 1.2 * cs.p_sz               # far enough from the inlet to spawn
    return cs, po, co, off, ent


@pytest.mark.parametrize("cid,grid,steps,outlet,inlet", [(1, (112, 48), 40, 0, 0), (3, (48, 12, 12), 8, 40, 60),
                                                         (2, (32, 8, 8), 4, 20, 30), (4, (96, 96), 3, 0, 0)])
def test_split_merge_bitwise(gpu_mod, oracle_mod, cid, grid, steps, outlet, inlet):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, po, co, off, ent = _event_state(M, O, cid, grid, steps, seed=cid, outlet=outlet, inlet=inlet)
    g = M.MPM(cs, PREC_FP64)
    o = O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(po)
        x.upload_cells(co)
        x.upload_lists(off, ent)
    g.Map_the_particle_to_tree()
    o.Map_the_particle_to_tree()
    g.Split_particle_fast()
    o.Split_particle_fast()
    g.sync()
    assert particles_bitwise_equal(g.download_particles(), o.download_particles()) == []
    gl, ol = g.download_cell_lists(), o.download_cell_lists()
    assert np.array_equal(gl[0], ol[0]) and np.array_equal(gl[1], ol[1])
    sg, so = g.stats(), o.stats()
    assert sg["n_split"] == so["n_split"] > 0
    assert (sg["n_inlet"], sg["n_outlet"], sg["n_affected"]) == (so["n_inlet"], so["n_outlet"], so["n_affected"])
    if inlet:
        assert sg["n_inlet"] > 0
    if outlet:
        assert sg["n_outlet"] > 0
    for it in range(4):
        g.Merge_particle_fast()
        o.Merge_particle_fast()
        g.sync()
        assert particles_bitwise_equal(g.download_particles(), o.download_particles()) == [], f"merge pass {it}"
        gl, ol = g.download_cell_lists(), o.download_cell_lists()
        assert np.array_equal(gl[0], ol[0]) and np.array_equal(gl[1], ol[1])
    sg, so = g.stats(), o.stats()
    assert sg["n_merge"] == so["n_merge"] > 0
    assert sg["n_affected"] == so["n_affected"]
    assert _lists_match(g, o) == 0


def test_canonical_order_invariants(gpu_mod, oracle_mod):
    """New particles are appended in parent order with increasing creation
    rank; removed ones leave the rest in order."""
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, po, co, off, ent = _event_state(M, O, 1, (112, 48), 20, seed=7, frac=0.05)
    g = M.MPM(cs, PREC_FP64)
    g.upload_particles(po)
    g.upload_cells(co)
    g.upload_lists(off, ent)
    g.Map_the_particle_to_tree()
    g.Split_particle_fast()
    q = g.download_particles()
    assert np.all(np.diff(q.seq.astype(np.int64)) > 0)
    assert q.n > po.n
    for _ in range(4):
        g.Merge_particle_fast()
    r = g.download_particles()
    assert np.all(np.diff(r.seq.astype(np.int64)) > 0)
    # volume is conserved by split (exact halvings) and merge (sum of pairs)
    assert abs(r.vol.sum() - po.vol.sum()) <= 1e-12 * po.vol.sum()
    # every live particle sits in exactly one cell list
    coff, cent = g.download_cell_lists()
    fluid = cent[cent >= 0]
    assert np.array_equal(np.sort(fluid), np.arange(r.n))


@pytest.mark.parametrize("cid,grid,steps", [(1, (112, 48), 40), (3, (48, 12, 12), 8)])
def test_step_merge_chain_bitwise(gpu_mod, oracle_mod, cid, grid, steps):
    """Whole steps from a state with split and merge candidates: the step's four
    merge passes run chained, and on the device a pass that follows one which
    merged nothing sweeps no slots.  Particles, cell lists and event counts
    still equal the oracle's bit for bit."""
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, po, co, off, ent = _event_state(M, O, cid, grid, steps, seed=10 + cid)
    g = M.MPM(cs, PREC_FP64)
    o = O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(po)
        x.upload_cells(co)
        x.upload_lists(off, ent)
    for s in range(2):
        g.advance(1)
        o.advance(1)
        g.sync()
        assert particles_bitwise_equal(g.download_particles(), o.download_particles()) == [], f"step {s + 1}"
        gl, ol = g.download_cell_lists(), o.download_cell_lists()
        assert np.array_equal(gl[0], ol[0]) and np.array_equal(gl[1], ol[1])
    sg, so = g.stats(), o.stats()
    for k in ("n_split", "n_merge", "n_inlet", "n_outlet"):
        assert sg[k] == so[k], k
    assert sg["n_merge"] > 0

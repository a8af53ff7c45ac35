"""MLS_P2G's skip of out-of-reach neighbour cells (mpm.cpp:274-382 visits all
3^d cells) rests on every particle lying in its bucket's cell from binning until
particles move, including the particles that split, inlet and merge add or
re-bin in between.  Direct method calls bin -> split -> 4 x merge -> P2G, with
split children and merge survivors crossing cell faces, must give the same cell
masses, volume fractions, phase flags and new-phase states with the skip as
with every neighbour cell visited."""
import numpy as np
import pytest

from tests.test_gpu_split_merge import _event_state

pytestmark = pytest.mark.gpu

KEYS = ("alph", "ph_state", "ph_state_b", "rho", "rhov", "E", "coef")


def _near_faces(cs, po, idx, frac=0.08):
    """Move the given particles to within frac * p_sz of the upper face of their
    cell along x, so that their split children land on both sides of it."""
    lo, dx = cs.box_l[0], cs.p_size[0]
    i = np.floor((po.coord[idx, 0] - lo) / dx)
    po.coord[idx, 0] = lo + (i + 1) * dx - frac * cs.p_sz


def _p2g_after_events(M, cs, po, co, off, ent, prec, skip):
    g = M.MPM(cs, prec)
    g.upload_particles(po)
    g.upload_cells(co)
    g.upload_lists(off, ent)
    assert g.tune("p2g_skip", skip) == skip
    g.Map_the_particle_to_tree()
    g.Split_particle_fast()
    for _ in range(cs.merge_iters):
        g.Merge_particle_fast()
    g.Refresh_membership()
    g.MLS_P2G()
    g.sync()
    st = g.stats()
    out = g.download_cells()
    g.close()
    return out, st


@pytest.mark.parametrize("cid,grid,steps", [(3, (48, 12, 12), 6), (1, (112, 48), 20), (2, (32, 8, 8), 4)])
@pytest.mark.parametrize("prec_name", ["FP64", "MIXED"])
def test_p2g_skip_matches_full_scan(gpu_mod, oracle_mod, cid, grid, steps, prec_name):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300 import abi
    prec = getattr(abi, "PREC_" + prec_name)
    cs, po, co, off, ent = _event_state(M, O, cid, grid, steps, seed=30 + cid, frac=0.04, inlet=20)
    vmax = cs.p_sz ** cs.dim * 1.6
    big = np.nonzero(po.vol > vmax)[0]
    _near_faces(cs, po, big[: len(big) // 2])
    full, s_full = _p2g_after_events(M, cs, po, co, off, ent, prec, 0)
    skip, s_skip = _p2g_after_events(M, cs, po, co, off, ent, prec, 1)
    assert s_full["n_split"] > 0 and s_full["n_merge"] > 0 and s_full["n_inlet"] > 0
    for k in ("n_split", "n_merge", "n_inlet", "n_outlet", "n_particles"):
        assert s_full[k] == s_skip[k], k
    bad = [k for k in KEYS if getattr(full, k).tobytes() != getattr(skip, k).tobytes()]
    assert bad == [], bad

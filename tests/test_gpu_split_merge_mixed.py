"""Split_particle_fast / Merge_particle_fast on the mixed-precision path, which
stores particles in FP32 but decides and indexes in FP64 on the same kernels
(mpm.cpp:1036-1417, 1536-1706): on inputs that are exactly representable in
FP32, every call gives the oracle's events, partners, child order (creation
ranks), phases, cell-list order and stored neighbour lists bit for bit, and
its float fields within FP32 rounding of the oracle's FP64 results.  Each call
starts both sides from the same FP32-exact state."""
import numpy as np
import pytest

from tests.test_gpu_split_merge import _event_state, _lists_match

pytestmark = pytest.mark.gpu

EXACT = ("phase", "mark_in", "seq")
FLOATS = ("coord", "v", "rhov", "vol", "mass", "h", "P", "rho", "E", "c", "slope")
# FP32 storage of FP64 results: half an ulp of FP32 relative to each field's scale
TOL_F32 = 2 ** -23


def _fp32_exact(p):
    q = p.copy()
    for k in FLOATS + ("tv",):
        a = getattr(q, k)
        a[...] = a.astype(np.float32).astype(np.float64)
    return q


def _check_call(g, o, dim, what):
    pg, po = g.download_particles(), o.download_particles()
    assert pg.n == po.n, what
    for k in EXACT:
        assert np.array_equal(getattr(pg, k), getattr(po, k)), (what, k)
    for k in FLOATS:
        a, b = getattr(pg, k), getattr(po, k)
        if a.ndim == 2 and a.shape[1] == 3:
            a, b = a[:, :dim], b[:, :dim]
        scale = np.maximum(np.abs(b), np.abs(b).max() * 1e-30)
        if k in ("coord", "v", "rhov", "slope"):
            scale = np.maximum(np.abs(b), np.abs(b).max(axis=0, keepdims=True))
        err = np.abs(a - b) / np.where(scale > 0, scale, 1)
        assert err.max() <= 2 * TOL_F32, (what, k, float(err.max()))
    gl, ol = g.download_cell_lists(), o.download_cell_lists()
    assert np.array_equal(gl[0], ol[0]) and np.array_equal(gl[1], ol[1]), what
    return po


def _fresh(M, O, cs, p, c, off, ent):
    from pgdg_p2_gb300.abi import PREC_MIXED
    g, o = M.MPM(cs, PREC_MIXED), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(p)
        x.upload_cells(c)
        x.upload_lists(off, ent)
        x.Map_the_particle_to_tree()
    return g, o


@pytest.mark.parametrize("cid,grid,steps,outlet,inlet", [(1, (112, 48), 40, 0, 0), (3, (48, 12, 12), 8, 40, 60),
                                                         (2, (32, 8, 8), 4, 20, 30), (4, (96, 96), 3, 0, 0)])
def test_split_merge_mixed_bitwise_indexing(gpu_mod, oracle_mod, cid, grid, steps, outlet, inlet):
    M, O = gpu_mod, oracle_mod
    cs, po, co, off, ent = _event_state(M, O, cid, grid, steps, seed=40 + cid, outlet=outlet, inlet=inlet)
    p = _fp32_exact(po)
    g, o = _fresh(M, O, cs, p, co, off, ent)
    g.Split_particle_fast()
    o.Split_particle_fast()
    g.sync()
    ps = _check_call(g, o, cs.dim, "split")
    sg, so = g.stats(), o.stats()
    for k in ("n_split", "n_inlet", "n_outlet", "n_affected"):
        assert sg[k] == so[k], k
    assert so["n_split"] > 0
    assert _lists_match(g, o) == 0
    # each merge pass from the oracle's previous result, made FP32-exact on both sides
    oof, oent = o.download_lists()
    merged = 0
    for it in range(cs.merge_iters):
        q = _fp32_exact(ps)
        g, o = _fresh(M, O, cs, q, o.download_cells(), oof, oent)
        g.Merge_particle_fast()
        o.Merge_particle_fast()
        g.sync()
        ps = _check_call(g, o, cs.dim, f"merge pass {it}")
        sg, so = g.stats(), o.stats()
        assert sg["n_merge"] == so["n_merge"] and sg["n_affected"] == so["n_affected"], it
        merged += so["n_merge"]
        assert _lists_match(g, o) == 0, it
        oof, oent = o.download_lists()
    assert merged > 0

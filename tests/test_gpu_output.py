"""pgdg_output_plt (MPM::Output_plt_file, mpm_ini.cpp:832-980) against the
oracle's restatement: on the exact FP64 path both files equal the oracle's
byte for byte after stepping (the state, the flag-2 list sizes, the norms and
the %g text are all the same); on the mixed path every value lies within FP32
rounding of the oracle's and the list sizes agree but for candidates at the
2h boundary; a snapshot written asynchronously while the context steps on
equals the one written synchronously from the same state."""
import numpy as np
import pytest

from tests.plt_read import read_cell_table, read_particle_plt

pytestmark = pytest.mark.gpu


def _pair(M, O, cid, grid, prec):
    cs, p, c = M.make_case(cid, grid)
    g, o = M.MPM(cs, prec), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(p)
        x.upload_cells(c)
    return cs, g, o


@pytest.mark.parametrize("cid,grid,steps", [(3, (48, 12, 12), 6), (1, (112, 48), 20), (2, (32, 8, 8), 4),
                                            (4, (64, 64), 3)])
def test_exact_snapshot_equals_oracle(gpu_mod, oracle_mod, tmp_path, cid, grid, steps):
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, g, o = _pair(gpu_mod, oracle_mod, cid, grid, PREC_FP64)
    for x in (g, o):
        x.advance(steps)
    g.output_plt(tmp_path / "g.plt", tmp_path / "g.cells")
    o.output_plt(tmp_path / "o.plt", tmp_path / "o.cells")
    gb, ob = (tmp_path / "g.plt").read_bytes(), (tmp_path / "o.plt").read_bytes()
    if gb != ob:
        hg, dg = read_particle_plt(tmp_path / "g.plt")
        ho, do = read_particle_plt(tmp_path / "o.plt")
        bad = [k for k in do if not np.array_equal(dg[k], do[k])]
        raise AssertionError(("particle file differs", bad, hg["time"], ho["time"]))
    assert (tmp_path / "g.cells").read_bytes() == (tmp_path / "o.cells").read_bytes()


@pytest.mark.parametrize("cid,grid,steps", [(3, (48, 12, 12), 6), (1, (112, 48), 20)])
def test_mixed_snapshot_close_to_oracle(gpu_mod, oracle_mod, tmp_path, cid, grid, steps):
    from pgdg_p2_gb300.abi import PREC_MIXED
    cs, g, o = _pair(gpu_mod, oracle_mod, cid, grid, PREC_MIXED)
    # lock-step time steps (the oracle's), as the accuracy tests run
    for s in range(1, steps + 1):
        dt, mv = o.Set_timestep()
        g.Set_timestep()
        g.set_dt(dt)
        g.set_max_v(mv)
        for x in (g, o):
            x.set_iterate(s)
            x.MPM_run_simulation(s)
    g.output_plt(tmp_path / "g.plt", tmp_path / "g.cells")
    o.output_plt(tmp_path / "o.plt", tmp_path / "o.cells")
    hg, dg = read_particle_plt(tmp_path / "g.plt")
    ho, do = read_particle_plt(tmp_path / "o.plt")
    for k in ("names", "types", "zone", "imax", "ranges"):
        assert hg[k] == ho[k], k
    assert abs(hg["time"] - ho["time"]) <= 1e-12 * ho["time"]
    assert np.array_equal(dg["phase"], do["phase"])
    for k in ("x", "y", "z"):
        # positions against the box size (relative error is meaningless near 0)
        assert np.max(np.abs(dg[k] - do[k])) <= 1e-5 * max(np.abs(do[k]).max(), 1e-30), k
    # the state fields by relative L1 (the accuracy measure of the path; single
    # particles at the shock move by more than FP32 rounding)
    def l1(a, b):
        return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))
    errs = {k: l1(dg[k], do[k]) for k in ("vol", "rho", "P", "v", "tv")}
    # velocity components against the speed (a transverse component near zero
    # is rounding noise of the reference algorithm itself)
    vsum = max(np.abs(do["v"]).sum(), 1e-300)
    for k in ("vx", "vy"):
        errs[k] = float(np.abs(dg[k] - do[k]).sum() / vsum)
    print(errs)
    for k in ("vol", "rho", "P"):
        assert errs[k] <= 1e-4, (k, errs[k])
    for k in ("vx", "vy", "v", "tv"):
        assert errs[k] <= 1e-3, (k, errs[k])
    same = np.mean(dg["n_neighbor"] == do["n_neighbor"])
    assert same >= 0.99 and np.abs(dg["n_neighbor"] - do["n_neighbor"]).max() <= 4, same
    (g1, g2), rg = read_cell_table(tmp_path / "g.cells")
    (o1, o2), ro = read_cell_table(tmp_path / "o.cells")
    assert g1 == o1 and rg.shape == ro.shape
    assert np.array_equal(rg[:, :3], ro[:, :3])
    # phase fractions and the mixture quantities; slopes and limiters are not
    # compared (near-zero slopes are ratios of rounding noise)
    for col in (6, 7, 12, 13, 14):
        assert l1(rg[:, col], ro[:, col]) <= 1e-3, col


def test_async_snapshot_equals_sync(gpu_mod, tmp_path):
    """The asynchronous writer copies a snapshot: stepping on while it writes
    leaves the files equal to a synchronous write of the same state."""
    M = gpu_mod
    from pgdg_p2_gb300.abi import PREC_MIXED
    cs, p, c = M.make_case(3, (64, 16, 16))
    ctx = []
    for _ in range(2):
        g = M.MPM(cs, PREC_MIXED)
        g.tune("pst", 0)
        g.upload_particles(p)
        g.upload_cells(c)
        g.advance(5)
        ctx.append(g)
    a, b = ctx
    a.output_plt(tmp_path / "a.plt", tmp_path / "a.cells", async_write=True)
    a.advance(4)
    a.output_wait()
    b.output_plt(tmp_path / "b.plt", tmp_path / "b.cells")
    assert (tmp_path / "a.plt").read_bytes() == (tmp_path / "b.plt").read_bytes()
    assert (tmp_path / "a.cells").read_bytes() == (tmp_path / "b.cells").read_bytes()
    # and a second snapshot after the extra steps differs
    a.output_plt(tmp_path / "a2.plt", None)
    assert (tmp_path / "a2.plt").read_bytes() != (tmp_path / "a.plt").read_bytes()

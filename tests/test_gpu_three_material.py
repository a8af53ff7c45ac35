"""The three-material instance (FldNum = 3, Triple_point_3phase) on
libpgdg_gpu_f3.so, the same kernels built with -DPGDG_NFLD=3: the exact path
equals the three-material oracle bit for bit step after step, the device case
builder equals the uploaded case, the snapshot files equal the oracle's, and
the mixed path meets the accuracy gate of the two-material runs through the
interaction of the three materials."""
import numpy as np
import pytest

from tests.gpu_helpers import cells_bitwise_equal, conserved_l1, floor_gate, fp32_perturbed, particles_bitwise_equal

pytestmark = pytest.mark.gpu


def test_three_material_exact_steps_bitwise(gpu_mod, oracle_mod, tmp_path):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_FP64
    cs, p, c = M.make_case(5)
    g, o = M.MPM(cs, PREC_FP64), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(p)
        x.upload_cells(c)
    for s in range(24):
        for x in (g, o):
            x.advance(1)
        g.sync()
        assert particles_bitwise_equal(g.download_particles(), o.download_particles()) == [], f"step {s + 1}"
    assert cells_bitwise_equal(g.download_cells(), o.download_cells()) == []
    sg, so = g.stats(), o.stats()
    for k in ("n_split", "n_merge", "mgfm_calls", "mgfm_iters"):
        assert sg[k] == so[k], k
    assert so["mgfm_calls"] > 0
    tg, to = g.totals(), o.totals()
    assert tg.shape == (8,) and tg.tobytes() == to.tobytes()
    g.output_plt(tmp_path / "g.plt", tmp_path / "g.cells")
    o.output_plt(tmp_path / "o.plt", tmp_path / "o.cells")
    assert (tmp_path / "g.plt").read_bytes() == (tmp_path / "o.plt").read_bytes()
    assert (tmp_path / "g.cells").read_bytes() == (tmp_path / "o.cells").read_bytes()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_three_material_device_case(gpu_mod, prec):
    M = gpu_mod
    cs, p, c = M.make_case(5)
    up, dev = M.MPM(cs, prec), M.MPM(cs, prec)
    up.upload_particles(p)
    up.upload_cells(c)
    dev.case_build(5, 0)
    assert particles_bitwise_equal(dev.download_particles(), up.download_particles()) == []
    assert cells_bitwise_equal(dev.download_cells(), up.download_cells()) == []


def test_three_material_mixed_accuracy(gpu_mod, oracle_mod):
    """150 lock-step steps (t ~ 0.5); relative L1 per conserved variable within
    max(1e-3, 3x the oracle's own L1 under FP32-sized input perturbation)."""
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300.abi import PREC_MIXED
    cs, p, c = M.make_case(5)
    o, ob, g = O.Oracle(cs), O.Oracle(cs), M.MPM(cs, PREC_MIXED)
    o.upload_particles(p)
    ob.upload_particles(fp32_perturbed(p))
    g.upload_particles(p)
    for x in (o, ob, g):
        x.upload_cells(c)
    for s in range(1, 151):
        dt, mv = o.Set_timestep()
        for x in (ob, g):
            x.Set_timestep()
            x.set_dt(dt)
            x.set_max_v(mv)
        for x in (o, ob, g):
            x.set_iterate(s)
            x.MPM_run_simulation(s)
    g.sync()
    co = o.download_cells()
    floor, _ = conserved_l1(cs, ob.download_cells(), co)
    per, mom = conserved_l1(cs, g.download_cells(), co)
    print({"l1": per, "floor": floor, "momentum": mom, "oracle": o.stats(), "gpu": g.stats()})
    assert not floor_gate(per, floor, 1e-3, 3.0), (per, floor)
    so = o.stats()
    assert so["mgfm_calls"] > 0 and so["n_split"] + so["n_merge"] > 0
    tg, to = g.totals(), o.totals()
    assert np.all(np.abs(tg - to) <= 1e-3 * np.abs(to)), (tg, to)


@pytest.mark.parametrize("prec_name", ["MIXED", "FP64_FMA"])
def test_particle_on_a_wall_stays_finite(gpu_mod, prec_name):
    """Bound_pen's 0.02 / dis (particle_flow.cpp:587-622) is infinite for a
    particle exactly on a wall, which FP32 coordinates reach far more often
    than FP64 ones (a three-material run met one after 110 steps); the
    reduced-precision paths push it off the wall by at most p_sz / 2."""
    M = gpu_mod
    from pgdg_p2_gb300 import abi
    cs, p, c = M.make_case(1)
    on = [0, 1, 2]
    p.coord[on[0], 1] = 0.0            # bottom wall
    p.coord[on[1], 0] = 0.0            # left wall
    top = int(np.argmax(p.coord[:, 1]))
    p.coord[top, 1] = 3.0              # top wall
    g = M.MPM(cs, getattr(abi, "PREC_" + prec_name))
    g.upload_particles(p)
    g.upload_cells(c)
    g.advance(3)
    g.sync()
    q = g.download_particles()
    assert np.all(np.isfinite(q.coord[:, :2])) and np.all(np.isfinite(q.rho)) and np.all(np.isfinite(q.E))
    assert q.coord[:, 1].min() >= 0.0 and q.coord[:, 1].max() <= 3.0 and q.coord[:, 0].min() >= 0.0

"""MPM::Initialize_case on the device (pgdg_case_build): the particles and cells
it writes in place equal, bit for bit, the host builder's arrays uploaded
through the C ABI, on every workload and precision; and steps from either
start give the same state."""
import pytest

from tests.gpu_helpers import cells_bitwise_equal, particles_bitwise_equal

pytestmark = pytest.mark.gpu

KEYS = ("rho", "rhov", "E", "c", "ac", "alph", "coef", "v", "P", "ph_state", "ph_state_b", "used", "lim_u", "g_v",
        "dcoef")


@pytest.mark.parametrize("cid,grid,seed", [(1, (112, 48), 0), (1, (56, 24), 77), (2, (32, 8, 8), 0),
                                           (3, (48, 12, 12), 0), (4, (64, 64), 0)])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_device_case_equals_uploaded_case(gpu_mod, cid, grid, seed, prec):
    M = gpu_mod
    cs, p, c = M.make_case(cid, grid, seed)
    up, dev = M.MPM(cs, prec), M.MPM(cs, prec)
    up.upload_particles(p)
    up.upload_cells(c)
    dev.case_build(cid, seed)
    assert particles_bitwise_equal(dev.download_particles(), up.download_particles()) == []
    assert cells_bitwise_equal(dev.download_cells(), up.download_cells(), KEYS) == []
    for g in (up, dev):
        g.tune("pst", 0)
        g.advance(2)
        g.sync()
    assert particles_bitwise_equal(dev.download_particles(), up.download_particles()) == []
    assert cells_bitwise_equal(dev.download_cells(), up.download_cells()) == []
    assert dev.stats()["n_particles"] == up.stats()["n_particles"] == p.n

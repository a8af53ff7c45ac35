"""pgdg_advance with captured CUDA graphs of whole steps against the same
steps run eagerly: bit-identical particle and cell state."""
import pytest

from tests.gpu_helpers import cells_bitwise_equal, particles_bitwise_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cid,grid,prec", [(1, (112, 48, 1), 0), (3, (48, 12, 12), 0), (3, (48, 12, 12), 1),
                                           (4, (64, 64, 1), 1)])
def test_graph_steps_equal_eager_steps(gpu_mod, cid, grid, prec):
    M = gpu_mod
    cs, p, c = M.make_case(cid, grid)
    out = []
    chosen = -1
    for graphs in (False, True):
        g = M.MPM(cs, prec)
        g.set_graphs(graphs)
        if chosen >= 0:
            # the shifting variants agree only to rounding: bitwise comparison
            # needs the variant the eager run's tuner chose
            g.tune("pst", chosen)
        g.upload_particles(p)
        g.upload_cells(c)
        g.advance(2)            # first iteration and tuning run eagerly
        g.advance(7)            # 2 x 3 steps from graphs + 1 eager step when enabled
        g.sync()
        chosen = g.tune("pst")
        out.append((g.download_particles(), g.download_cells(), g.stats()))
        g.close()
    (pa, ca, sa), (pb, cb, sb) = out
    assert particles_bitwise_equal(pb, pa) == []
    assert cells_bitwise_equal(cb, ca) == []
    assert sa["iterate_num"] == sb["iterate_num"] == 9

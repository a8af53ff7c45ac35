"""pgdg_advance with captured CUDA graphs of whole steps against the same
steps run eagerly: bit-identical particle and cell state, including the
learned mixed path, whose interface batch is sized on the device."""
import pytest

from tests.gpu_helpers import cells_bitwise_equal, particles_bitwise_equal

pytestmark = pytest.mark.gpu


def _run(M, S, cs, p, c, prec, graphs, chosen, learned, iface_cap=-1, steps=(2, 7)):
    g = M.MPM(cs, prec)
    net = None
    if learned:
        net = S.Surrogate(S.load_default(), tc=True)
        g.set_surrogate(net)
    if iface_cap >= 0:
        g.tune("iface_cap", iface_cap)
    g.set_graphs(graphs)
    if chosen >= 0:
        # the shifting variants agree only to rounding: bitwise comparison
        # needs the variant the eager run's tuner chose
        g.tune("pst", chosen)
    g.upload_particles(p)
    g.upload_cells(c)
    for n in steps:
        g.advance(n)
    g.sync()
    out = (g.download_particles(), g.download_cells(), g.stats(), g.tune("pst"))
    g.close()
    if net is not None:
        net.close()
    return out


@pytest.mark.parametrize("cid,grid,prec,learned", [(1, (112, 48, 1), 0, False), (3, (48, 12, 12), 0, False),
                                                   (3, (48, 12, 12), 1, False), (4, (64, 64, 1), 1, False),
                                                   (3, (48, 12, 12), 1, True), (4, (64, 64, 1), 1, True)])
def test_graph_steps_equal_eager_steps(gpu_mod, cid, grid, prec, learned):
    M = gpu_mod
    from pgdg_p2_gb300 import surrogate as S
    cs, p, c = M.make_case(cid, grid)
    # first iteration and tuning run eagerly; then 2 x 3 steps from graphs + 1 eager step when enabled
    pa, ca, sa, chosen = _run(M, S, cs, p, c, prec, False, -1, learned)
    pb, cb, sb, _ = _run(M, S, cs, p, c, prec, True, chosen, learned)
    # one call from the start: its first graph is captured right after the
    # eager first iterations
    pc, cc, sc, _ = _run(M, S, cs, p, c, prec, True, chosen, learned, steps=(9,))
    assert particles_bitwise_equal(pc, pa) == [] and cells_bitwise_equal(cc, ca) == []
    assert particles_bitwise_equal(pb, pa) == []
    assert cells_bitwise_equal(cb, ca) == []
    assert sa["iterate_num"] == sb["iterate_num"] == 9
    if learned:
        assert sa["mgfm_calls"] == sb["mgfm_calls"] > 0 and sa["mgfm_iters"] == sb["mgfm_iters"]


def test_queue_overflow_runs_the_inline_solve(gpu_mod):
    """A learned context whose interface queue holds a single problem solves
    every stage inline from the reference's seed: bit for bit the mixed path
    without the queue, eager and from graphs."""
    M = gpu_mod
    from pgdg_p2_gb300 import surrogate as S
    from pgdg_p2_gb300.abi import PREC_MIXED
    cs, p, c = M.make_case(3, (48, 12, 12))
    pa, ca, sa, chosen = _run(M, S, cs, p, c, PREC_MIXED, False, -1, False)
    for graphs in (False, True):
        pb, cb, sb, _ = _run(M, S, cs, p, c, PREC_MIXED, graphs, chosen, True, iface_cap=1)
        assert particles_bitwise_equal(pb, pa) == [], graphs
        assert cells_bitwise_equal(cb, ca) == [], graphs
        assert sb["mgfm_calls"] == sa["mgfm_calls"] and sb["mgfm_iters"] == sa["mgfm_iters"], graphs

"""The premise of the device's skipped merge passes, checked on the CPU oracle:
a Merge_particle_fast pass (mpm.cpp:1536-1706) that follows a pass which merged
nothing finds the same partners on the same state and leaves particles, cell
lists and stored neighbour lists bit for bit unchanged."""
import numpy as np

from tests.gpu_helpers import particles_bitwise_equal


def test_pass_after_quiet_pass_changes_nothing(oracle_mod):
    from pgdg_p2_gb300 import mpm as M
    from tests.test_gpu_split_merge import _event_state
    O = oracle_mod
    cs, po, co, off, ent = _event_state(M, O, 1, (112, 48), 40, seed=1)
    o = O.Oracle(cs)
    o.upload_particles(po)
    o.upload_cells(co)
    o.upload_lists(off, ent)
    o.Map_the_particle_to_tree()
    o.Split_particle_fast()
    merged = []
    for _ in range(8):
        before = o.stats()["n_merge"]
        o.Merge_particle_fast()
        merged.append(o.stats()["n_merge"] - before)
        if merged[-1] == 0:
            break
    assert merged[0] > 0 and merged[-1] == 0, merged
    p0, l0, n0 = o.download_particles(), o.download_cell_lists(), o.download_lists()
    o.Merge_particle_fast()
    p1, l1, n1 = o.download_particles(), o.download_cell_lists(), o.download_lists()
    assert particles_bitwise_equal(p1, p0) == []
    assert all(np.array_equal(a, b) for a, b in zip(l1, l0))
    assert all(np.array_equal(a, b) for a, b in zip(n1, n0))
    assert o.stats()["n_merge"] == sum(merged)

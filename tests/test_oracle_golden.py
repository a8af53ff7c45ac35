"""The oracle reproduces its committed golden digests (tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from tests.golden.make_golden import CASES, digest_cells, digest_particles, run_case, summary

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))


@pytest.mark.parametrize("name,cid,grid,steps", CASES)
def test_oracle_digest(name, cid, grid, steps):
    g = GOLD[name]
    cs, p0, o = run_case(cid, grid, steps, g["case"])
    assert digest_particles(p0, cs.dim) == g["initial_particles"]
    p, c = o.download_particles(), o.download_cells()
    assert summary(p, c, cs.dim) == pytest.approx(g["summary"], rel=1e-12)
    assert digest_particles(p, cs.dim) == g["particles"]
    assert digest_cells(c) == g["cells"]


def test_mgfm_known_values():
    from oracle import oracle as O
    k = json.load(open(os.path.join(HERE, "golden", "mgfm_known.json")))
    out, it = O.mgfm_batched(np.array(k["in6"]), np.array(k["mat2"], np.int8), np.array(k["gamma"]),
                             np.array(k["pinf"]), 0)
    assert np.array_equal(out, np.array(k["out3"]))
    assert np.array_equal(it, np.array(k["iters"]))

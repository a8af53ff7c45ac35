"""The neighbour cells P2G skips while the bins are fresh (p2g_skip in k_grid.cu),
restated in Python: a cell whose box, shrunk by 1e-4 of a cell, stays beyond the
cut radius 1.5 p_sz of the centre cell's centre is skipped.  Particles lie in
their cell up to rounding, so no particle of a skipped cell may be within the
cut radius; on the 8-per-cell lattice the eight corner cells are the ones."""
import itertools

import numpy as np
import pytest


def skip_mask(ps, p_sz, dim):
    cut = 1.5 * p_sz
    mask = 0
    for code in range(8):
        if dim == 2 and code & 4:
            continue
        g2 = 0.0
        for d in range(dim):
            if code & (1 << d):
                g = 0.5 * ps[d] * (1.0 - 1e-4)
                g2 += g * g
        if g2 > cut * cut:
            mask |= 1 << code
    return mask


@pytest.mark.parametrize("dim,ps,p_sz", [(3, (1.0, 1.0, 1.0), 0.5), (3, (1.0, 1.2, 0.9), 0.5),
                                         (2, (1.0, 1.0, 1.0), 0.5), (3, (1.0, 1.0, 1.0), 0.6)])
def test_skipped_cells_hold_no_contributor(dim, ps, p_sz):
    mask = skip_mask(ps, p_sz, dim)
    cut = 1.5 * p_sz
    rng = np.random.default_rng(7)
    centre = np.array([0.5 * ps[d] for d in range(dim)])
    for off in itertools.product((-1, 0, 1), repeat=dim):
        code = sum(1 << d for d in range(dim) if off[d] != 0)
        if not (mask >> code) & 1:
            continue
        lo = np.array([off[d] * ps[d] for d in range(dim)])
        # particles anywhere in the neighbour cell, its faces and corners included,
        # rounded to FP32 as the mixed path stores them
        pts = lo + rng.uniform(0.0, 1.0, (20000, dim)) * np.array(ps[:dim])
        corners = np.array([[lo[d] + (ps[d] if (c >> d) & 1 else 0.0) for d in range(dim)]
                            for c in range(1 << dim)])
        pts = np.vstack([pts, corners]).astype(np.float32).astype(np.float64)
        dist = np.sqrt(((pts - centre) ** 2).sum(1))
        assert dist.min() > cut, (off, dist.min(), cut)


def test_lattice_skips_exactly_the_corners():
    assert skip_mask((1.0, 1.0, 1.0), 0.5, 3) == 1 << 7
    assert skip_mask((1.0, 1.0, 1.0), 0.5, 2) == 0

"""The per-stage row sort of the shifting kernel (k_rs_cells / k_rs_rows /
k_rs_rank in k_g2p.cu), restated in Python over one row of cells.

Each cell's entries are sorted into a run.  An entry's rank in the row is its
place in its run plus, for the two neighbouring runs, the entries on the other
side of its key.  The prefix maxima and suffix minima of the run keys confirm
that no farther run interleaves; otherwise every run of the row is counted.
The tests drive rows with small drift (the path the device takes) and with
entries displaced by up to 2.5 cells (the full-count fallback), and check that
the ranks form a permutation that sorts the row by key."""
import numpy as np
import pytest


def row_key(z, slot):
    """(order-preserving integer image of the float32 coordinate, slot), as RowKey<float>."""
    i = int(np.float32(z).view(np.int32))
    k = i if i >= 0 else i ^ 0x7FFFFFFF
    return ((k & 0xFFFFFFFF) ^ 0x80000000) << 32 | slot


def rank_row(cells):
    """cells: list of lists of (z, slot) per cell in row order -> ranks per cell,
    first and last rank per cell, and whether the fallback was taken."""
    runs = [sorted(c, key=lambda e: row_key(*e)) for c in cells]
    keys = [[row_key(*e) for e in r] for r in runs]
    nr = len(runs)
    lowest, highest = -1, 1 << 70
    kmin = [k[0] if k else highest for k in keys]
    kmax = [k[-1] if k else lowest for k in keys]
    off, pmaxk, smink = [], [], [0] * nr
    acc, mx = 0, lowest
    for k in range(nr):
        off.append(acc)
        acc += len(runs[k])
        mx = max(mx, kmax[k])
        pmaxk.append(mx)
    mn = highest
    for k in range(nr - 1, -1, -1):
        mn = min(mn, kmin[k])
        smink[k] = mn

    def count_less(j, key):
        if not keys[j] or key < kmin[j]:
            return 0
        if kmax[j] < key:
            return len(keys[j])
        return int(np.searchsorted(np.array(keys[j], dtype=object), key))

    ranks, first, last, fell = [], [], [], False
    for k in range(nr):
        rk = []
        for r, key in enumerate(keys[k]):
            rank = off[k] + r
            if k >= 1:
                rank -= len(keys[k - 1]) - count_less(k - 1, key)
            if k + 1 < nr:
                rank += count_less(k + 1, key)
            far_ok = (k < 2 or pmaxk[k - 2] < key) and (k + 2 >= nr or key < smink[k + 2])
            if not far_ok:
                fell = True
                rank = r + sum(count_less(j, key) for j in range(nr) if j != k)
            rk.append(rank)
        ranks.append(rk)
        first.append(rk[0] if rk else None)
        last.append(rk[-1] if rk else None)
    return runs, keys, ranks, first, last, fell


def make_row(rng, nr, drift):
    cells, slot = [], 0
    for k in range(nr):
        n = int(rng.integers(0, 13))
        c = []
        for _ in range(n):
            z = k + rng.uniform(0.0, 1.0)
            if drift and rng.uniform() < 0.1:
                z += rng.uniform(-drift, drift)
            c.append((float(np.float32(z)), slot))
            slot += 1
        cells.append(c)
    return cells


@pytest.mark.parametrize("seed,nr,drift", [(1, 8, 0.0), (2, 12, 0.4), (3, 20, 0.9), (4, 12, 2.5), (5, 96, 2.5)])
def test_row_ranks_sort_the_row(seed, nr, drift):
    rng = np.random.default_rng(seed)
    cells = make_row(rng, nr, drift)
    runs, keys, ranks, first, last, fell = rank_row(cells)
    flat_keys = [key for k in keys for key in k]
    flat_ranks = [r for rk in ranks for r in rk]
    m = len(flat_keys)
    assert sorted(flat_ranks) == list(range(m))
    order = [None] * m
    for key, r in zip(flat_keys, flat_ranks):
        order[r] = key
    assert order == sorted(flat_keys)
    for k in range(nr):
        if ranks[k]:
            assert first[k] == min(ranks[k]) and last[k] == max(ranks[k])
    if drift > 2:
        assert fell, "the displaced entries should take the full count"


def test_key_order_matches_float_order_with_ties():
    zs = np.float32([-2.5, -0.0, 0.0, 1e-30, 3.25, 3.25])
    keys = [row_key(float(z), s) for s, z in enumerate(zs)]
    assert keys == sorted(keys)
    assert row_key(3.25, 4) < row_key(3.25, 5)

"""Generate the golden fixtures in this directory (run from the repository root).

The reference ships no tests, fixtures or golden vectors, so the fixtures pin the
CPU oracle itself: for small instances of each workload they record the case
parameters (so no machine recomputes them), and SHA-256 digests plus a few
summary numbers of the full FP64 particle and cell state after a number of
steps.  The oracle is evaluated without FMA contraction and with a correctly
rounded cube root, so the digests are the same on x86_64 and aarch64; the
exact-order FP64 GPU path reproduces them bit for bit.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = [
    # name, config id, grid, steps
    ("c1_triple_point_112x48", 1, (112, 48, 1), 30),
    ("c2_cylinder_32x8x8", 2, (32, 8, 8), 4),
    ("c3_sphere_48x12x12", 3, (48, 12, 12), 6),
    ("c4_undex_96x96", 4, (96, 96, 1), 5),
]


def digest_particles(p, dim):
    h = hashlib.sha256()
    for k in p.NAMES:
        a = getattr(p, k)
        if k in ("coord", "v", "tv", "rhov"):
            a = a[:, :dim]
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def digest_cells(c):
    h = hashlib.sha256()
    for k in ("rho", "rhov", "E", "c", "ac", "alph", "coef", "v", "P", "ph_state", "ph_state_b", "used"):
        h.update(np.ascontiguousarray(getattr(c, k)).tobytes())
    return h.hexdigest()


def summary(p, c, dim):
    return {"n": int(p.n), "mass": float((p.rho * p.vol).sum()), "energy": float((p.E * p.vol).sum()),
            "max_seq": int(p.seq.max()) if p.n else -1, "cell_mass": float((c.alph * c.rho).sum())}


def run_case(cid, grid, steps, case_dict=None):
    from oracle import oracle as O
    from pgdg_p2_gb300 import mpm as M
    from pgdg_p2_gb300.abi import pgdg_case
    cs = pgdg_case.from_dict(case_dict) if case_dict else M.case_setup(cid, grid)
    p = M.case_particles(cs, cid)
    c = M.case_cells(cs)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    o.advance(steps)
    return cs, p, o


def main():
    from oracle import oracle as O
    O.set_threads(os.cpu_count())
    out = {}
    for name, cid, grid, steps in CASES:
        cs, p0, o = run_case(cid, grid, steps)
        p, c = o.download_particles(), o.download_cells()
        st = o.stats()
        out[name] = {"config": cid, "grid": list(grid), "steps": steps, "case": cs.to_dict(),
                     "initial_particles": digest_particles(p0, cs.dim),
                     "particles": digest_particles(p, cs.dim), "cells": digest_cells(c),
                     "summary": summary(p, c, cs.dim),
                     "events": {k: st[k] for k in ("n_split", "n_merge", "n_inlet", "n_outlet", "mgfm_calls")}}
        print(name, out[name]["summary"], out[name]["events"])
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump(out, f, indent=1)
    # MGFM known values: seeded stiffened-gas problems (the micro-benchmark's distribution)
    rng = np.random.default_rng(5)
    n = 64
    inp, mat = mgfm_inputs(rng, n)
    gam = np.array([1.4, 1.648, 7.15, 2.0])
    pinf = np.array([0.0, 0.0, 3.309e8, 0.0])
    res, it = O.mgfm_batched(inp, mat, gam, pinf, 0)
    with open(os.path.join(HERE, "mgfm_known.json"), "w") as f:
        json.dump({"in6": inp.tolist(), "mat2": mat.tolist(), "gamma": gam.tolist(), "pinf": pinf.tolist(),
                   "out3": res.tolist(), "iters": it.tolist()}, f)


def mgfm_inputs(rng, n):
    """Log-uniform densities on [1e-2, 1e3], pressure ratio log-uniform on [1e-3, 1e4]
    around the base pressure 1e5 (sides swapped with probability 1/2), normal
    velocities uniform on [-500, 500], material pairs from {air, He, water, gas}^2."""
    rl = 10 ** rng.uniform(-2, 3, n)
    rr = 10 ** rng.uniform(-2, 3, n)
    ratio = 10 ** rng.uniform(-3, 4, n)
    pl = np.full(n, 1e5)
    pr = 1e5 * ratio
    sw = rng.random(n) < 0.5
    pl[sw], pr[sw] = pr[sw].copy(), pl[sw].copy()
    ul = rng.uniform(-500, 500, n)
    ur = rng.uniform(-500, 500, n)
    mat = rng.integers(0, 4, (n, 2)).astype(np.int8)
    return np.stack([ul, ur, pl, pr, rl, rr], 1), mat


if __name__ == "__main__":
    main()

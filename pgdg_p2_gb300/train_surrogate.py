"""Train the MGFM seed surrogate on the GPU and write its parameters.

    python -m pgdg_p2_gb300.train_surrogate --out pgdg_p2_gb300/weights/mgfm_seed.npy

Training problems: the interface Riemann problems the mixed step itself queues
on the four synthetic workloads (triple point, cylinder, sphere, underwater
explosion; recorded once per step through the interface queue), plus the
batched micro-benchmark's distribution drawn from a different stream (seed 99)
than the one it is evaluated on (seed 5).  Targets are exact roots by
bisection; problems without a positive root are left out.  A JSON report of the
loss history and of the Newton iterations (plain seed, closed-form baseline
seed alone, learned seed) is written next to the parameters.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from . import mpm as M
from . import surrogate as S
from .abi import PREC_MIXED

SOLVER_CASES = [(3, (96, 24, 24), 40), (2, (64, 16, 16), 40), (1, (112, 48), 80), (4, (128, 128), 60)]


def solver_problems(log=print):
    """Interface problems of the mixed step on the synthetic workloads, with the
    material parameters of each problem (gl, pinf_l, gr, pinf_r) and the MGFM
    variant of the case's dimension."""
    rows = []
    for cid, grid, steps in SOLVER_CASES:
        cs, p, c = M.make_case(cid, grid)
        g = M.MPM(cs, PREC_MIXED)
        g.set_iface_queue(True)
        g.upload_particles(p)
        g.upload_cells(c)
        gam = np.array(cs.gamma[:2])
        pinf = np.array(cs.pinf[:2])
        n0 = 0
        for _ in range(steps):
            g.advance(1)
            in6, mat = g.iface_problems()
            if len(in6):
                rows.append((in6, gam[mat[:, 0]], pinf[mat[:, 0]], gam[mat[:, 1]], pinf[mat[:, 1]],
                             np.full(len(in6), cs.mgfm_variant)))
                n0 += len(in6)
        g.close()
        log(f"case {cid} {grid}: {n0} interface problems")
    return [np.concatenate([r[k] for r in rows]) for k in range(6)]


def as_material_table(in6, gl, il, gr, ir):
    """Express per-problem materials as indices into a table (what the device
    kernels take)."""
    pairs = np.stack([np.concatenate([gl, gr]), np.concatenate([il, ir])], 1)
    tab, inv = np.unique(pairs, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    n = len(in6)
    mat = np.stack([inv[:n], inv[n:]], 1).astype(np.int8)
    return mat, tab[:, 0].copy(), tab[:, 1].copy()


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=S.WEIGHTS)
    ap.add_argument("--steps", type=int, default=40000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--c5", type=int, default=1 << 21)
    ap.add_argument("--eval", type=int, default=1 << 20)
    a = ap.parse_args(argv)
    t0 = time.time()

    def log(msg):
        print(f"[{time.time() - t0:7.1f}s] {msg}", flush=True)

    # solver-generated problems
    sin6, sgl, sil, sgr, sir, svar = solver_problems(log)
    smat, sgam, spinf = as_material_table(sin6, sgl, sil, sgr, sir)
    # micro-benchmark distribution, training stream
    cin6, cmat = S.c5_problems(a.c5, seed=99)
    Xs, Ts = [], []
    for in6, mat, gam, pinf in ((sin6, smat, sgam, spinf), (cin6, cmat, S.C5_GAMMA, S.C5_PINF)):
        ps, us, has = S.exact_roots(in6, mat, gam, pinf)
        X, _, _ = S.features_np(in6[has], mat[has], gam, pinf)
        T = S.targets_np(in6[has], mat[has], gam, pinf, ps[has], us[has])
        ok = np.all(np.isfinite(X), 1) & np.all(np.isfinite(T), 1)
        Xs.append(X[ok])
        Ts.append(T[ok])
        log(f"{len(in6)} problems, {has.sum()} with a root, {ok.sum()} kept")
    # weight the solver's own problems up to half of the sample
    rep = max(1, len(Xs[1]) // max(len(Xs[0]), 1))
    X = np.concatenate([np.tile(Xs[0], (rep, 1)), Xs[1]])
    T = np.concatenate([np.tile(Ts[0], (rep, 1)), Ts[1]])
    log(f"training set {len(X)} ({len(Xs[0])} solver problems x {rep})")
    params, hist = S.train(X, T, steps=a.steps, batch=a.batch, lr=a.lr, seed=0, log=log)

    # evaluation: Newton iterations from the plain seed, the closed-form
    # baseline alone and the learned seed
    net = S.Surrogate(params)
    base = S.Surrogate(S.baseline_params())
    report = {"loss": hist, "train_rows": int(len(X)), "solver_rows": int(len(Xs[0]))}
    ein6, emat = S.c5_problems(a.eval, seed=5)
    evar = np.zeros(len(ein6), np.int32)
    for name, in6, mat, gam, pinf, var in (("c5", ein6, emat, S.C5_GAMMA, S.C5_PINF, evar),
                                           ("solver", sin6, smat, sgam, spinf, svar)):
        its = {}
        for key, h in (("plain", None), ("baseline", base), ("learned", net)):
            it = np.zeros(len(in6), np.int32)
            for v in (0, 1):
                m = var == v
                if m.any():
                    _, it[m] = S.mgfm_gpu(in6[m], mat[m], gam, pinf, h, v)
            its[key] = it
        conv = its["plain"] < 50
        r = {"n": int(len(in6)), "with_root": float(conv.mean())}
        for key, it in its.items():
            r[key + "_iters_root"] = float(it[conv].mean())
            r[key + "_iters_all"] = float(it.mean())
            r[key + "_iters_max_root"] = int(it[conv].max())
            r[key + "_fallbacks"] = int(((it >= 50) & conv).sum())
        report[name] = r
        log(f"{name}: {r}")
    net.close()
    base.close()
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    np.save(a.out, params.astype(np.float32))
    with open(os.path.splitext(a.out)[0] + "_report.json", "w") as f:
        json.dump(report, f, indent=1)
    log(f"wrote {a.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())

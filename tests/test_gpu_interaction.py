"""Accuracy of the GPU paths through the shock-bubble interaction, against the
FP64 oracle, under the unmodified gate

    L1(q) = sum_cells vol |q - q_oracle| / sum_cells vol |q_oracle|   (uniform vol)

per conserved variable q in {rho, rho u, rho v, (rho w), E} (phase-mixed
sum_s alph_s q_s).  The runs go past the contact of the shock with the bubble
(C3 at 96x24x24: shock at x = 1.0, sphere from x = 1.25, contact near step 96;
130 steps reach t ~ 0.24) and, for the triple point, through hundreds of splits
and merges.

The floor.  Each run also advances a second oracle from the same state with
every particle's energy moved by a relative 2^-24 (the rounding of an FP32
store), with a seeded random sign.  The L1 between the two oracles is the
reference algorithm's own sensitivity to rounding of that size: a path that
holds its state in FP32 cannot be expected to agree with the oracle more
closely.  It is far below 1e-3 for rho, rho u and E in most cases, but
  - the transverse momenta of the 3D cases (about 1/1700 of sum |rho u| at C3)
    reach 1e-2..5e-2 (even one FP64 ulp does that);
  - the triple point after its particles start to split and merge reaches
    2e-3..3e-2;
  - the underwater explosion reaches 3e-3..4e-3 in momentum: the limiter's
    positivity probe and slope ratios switch at the bubble interface where it
    crosses the symmetry lines, and FP32-sized changes move those switches.
The gate is therefore

    L1_path(q) <= max(1e-3, FLOOR_FACTOR * L1_floor(q))

with both numbers and the momentum-magnitude-normalised error reported for
every variable.  The plain FP64 GPU path (FMA contraction) is held to the same
gate, as the yardstick the mixed path is matched against."""
import json
import os

import pytest

from tests.gpu_helpers import conserved_l1, floor_gate, fp32_perturbed

pytestmark = pytest.mark.gpu

TOL = 1e-3
FLOOR_FACTOR = 3.0
OUT = os.environ.get("PGDG_ACCURACY_LOG")

# (config, grid, steps, checkpoints)
CASES = [(3, (96, 24, 24), 130, (100, 130)), (2, (64, 16, 16), 130, (65, 130)), (1, (112, 48), 200, (100, 200)),
         (4, (128, 128), 120, (60, 120))]


@pytest.mark.parametrize("cid,grid,steps,checks", CASES)
def test_accuracy_through_interaction(gpu_mod, oracle_mod, cid, grid, steps, checks):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300 import surrogate as S
    from pgdg_p2_gb300.abi import PREC_FP64_FMA, PREC_MIXED
    cs, p, c = M.make_case(cid, grid)
    o, ob = O.Oracle(cs), O.Oracle(cs)
    paths = {"mixed": M.MPM(cs, PREC_MIXED), "learned": M.MPM(cs, PREC_MIXED), "fp64": M.MPM(cs, PREC_FP64_FMA)}
    params = S.load_default()
    assert params is not None, "trained weights missing"
    net = S.Surrogate(params, tc=True)
    paths["learned"].set_surrogate(net)
    o.upload_particles(p)
    ob.upload_particles(fp32_perturbed(p))
    for x in (o, ob, *paths.values()):
        x.upload_cells(c)
    for g in paths.values():
        g.upload_particles(p)
    report = []
    for s in range(1, steps + 1):
        dt, mv = o.Set_timestep()
        for x in (ob, *paths.values()):
            x.Set_timestep()
            x.set_dt(dt)
            x.set_max_v(mv)
        for x in (o, ob, *paths.values()):
            x.set_iterate(s)
            x.MPM_run_simulation(s)
        if s not in checks:
            continue
        co = o.download_cells()
        floor, _ = conserved_l1(cs, ob.download_cells(), co)
        rec = {"config": cid, "grid": list(grid), "step": s, "floor": floor, "oracle_stats": o.stats()}
        for name, g in paths.items():
            g.sync()
            per, mom = conserved_l1(cs, g.download_cells(), co)
            rec[name] = {"l1": per, "momentum_over_sum_abs_rho_u": mom, "stats": g.stats()}
        report.append(rec)
        print(json.dumps(rec))
        for name in paths:
            bad = floor_gate(rec[name]["l1"], floor, TOL, FLOOR_FACTOR)
            assert not bad, (name, s, bad)
    if OUT:
        with open(OUT, "a") as fh:
            for r in report:
                fh.write(json.dumps(r) + "\n")
    net.close()
    # the runs cover the regime the gate is about: multi-iteration interface
    # solves in every case; splits and merges in the triple point
    so = report[-1]["oracle_stats"]
    assert so["mgfm_iters"] > 1.2 * so["mgfm_calls"], so
    if cid == 1:
        assert so["n_split"] > 100 and so["n_merge"] > 100, so
        for name in paths:
            sg = report[-1][name]["stats"]
            assert sg["n_split"] > 100 and sg["n_merge"] > 100, (name, sg)

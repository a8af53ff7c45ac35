"""Shared helpers of the GPU parity tests."""
import numpy as np

FLOAT_FIELDS3 = ("coord", "v", "tv", "rhov")


def particles_bitwise_equal(pg, po):
    """Field names whose bytes differ between two particle sets (empty when equal)."""
    if pg.n != po.n:
        return ["count"]
    bad = []
    for k in pg.NAMES:
        a, b = getattr(pg, k), getattr(po, k)
        if k in FLOAT_FIELDS3:
            a, b = a[:, :pg.dim], b[:, :pg.dim]
        if a.tobytes() != b.tobytes():
            bad.append(k)
    return bad


def cells_bitwise_equal(cg, co, keys=("rho", "rhov", "E", "c", "ac", "alph", "coef", "v", "P", "ph_state",
                                      "ph_state_b", "used")):
    return [k for k in keys if getattr(cg, k).tobytes() != getattr(co, k).tobytes()]


def conserved_l1(cs, cg, co):
    """Relative L1 per conserved variable of the phase-mixed cell averages,
    sum |q - q_ref| / sum |q_ref|, and for the momentum components also the
    error normalised by the momentum magnitude sum |rho u|."""
    U = cs.dim + 2
    per, mom = [], []
    mag = sum(np.abs((co.alph * co.coef[:, :, 1 + k, 0]).sum(1)) for k in range(cs.dim)).sum()
    for u in range(U):
        qg = (cg.alph * cg.coef[:, :, u, 0]).sum(1)
        qo = (co.alph * co.coef[:, :, u, 0]).sum(1)
        per.append(float(np.abs(qg - qo).sum() / max(np.abs(qo).sum(), 1e-300)))
        if 1 <= u <= cs.dim:
            mom.append(float(np.abs(qg - qo).sum() / max(mag, 1e-300)))
    return per, mom


def fp32_perturbed(p, seed=12345):
    """Particles with every energy scaled by 1 +- 2^-24 (seeded random signs):
    the size of rounding an FP64 value to FP32."""
    q = p.copy()
    sign = np.random.default_rng(seed).choice([-1.0, 1.0], size=q.E.shape)
    q.E[:] = q.E * (1.0 + sign * 2.0 ** -24)
    return q


def floor_gate(per, floor, tol=1e-3, factor=3.0):
    """Variables whose relative L1 exceeds max(tol, factor * floor), where floor
    is the oracle's own L1 under FP32-sized perturbation of its input."""
    return [(v, e, f) for v, (e, f) in enumerate(zip(per, floor)) if not e <= max(tol, factor * f)]

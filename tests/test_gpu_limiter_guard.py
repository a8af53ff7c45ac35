"""Calculate_limiter's ratio |u_min / (dU + 1e-20)| (mpm.cpp:392-738) has a zero
denominator when a negative slope increment dU equals -1e-20 in the working
precision.  In FP64 that takes an exact coincidence; in FP32 a slope of
1e-20 / dr is enough, and one turned up at the symmetry plane z = 0 of the
shock-bubble case at 384x96x96 after 289 steps, where the boundary form of
the limiter turned the infinite ratio into NaN and the NaN spread to the
cell's particles.  The reduced-precision paths cap the ratio; the limiter they
return for such a cell is finite and equal to the oracle's, whose FP64
denominator is not zero."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _slope_hitting(dz):
    """An FP32 slope s with fl32(s * dz) == fl32(-1e-20)."""
    target = np.float32(-1e-20)
    s = np.float32(target / dz)
    for _ in range(64):
        prod = np.float32(s * dz)
        if prod == target:
            return s
        s = np.nextafter(s, np.float32(-np.inf) if prod > target else np.float32(np.inf), dtype=np.float32)
    raise AssertionError("no slope found")


@pytest.mark.parametrize("prec_name", ["MIXED", "FP64_FMA"])
def test_zero_denominator_gives_finite_limiter(gpu_mod, oracle_mod, prec_name):
    M, O = gpu_mod, oracle_mod
    from pgdg_p2_gb300 import abi
    cs, p, c = M.make_case(3, (48, 12, 12))
    o0 = O.Oracle(cs)
    o0.upload_particles(p)
    o0.upload_cells(c)
    o0.advance(2)
    ps, cst = o0.download_particles(), o0.download_cells()
    off, ent = o0.download_lists()
    grid = (48, 12, 12)
    ijk = (10, 5, 0)
    ci = np.ravel_multi_index(ijk, grid)
    nb = np.ravel_multi_index((ijk[0] + 1, ijk[1], ijk[2]), grid)
    assert cst.used[ci] and cst.alph[ci, 0] == 1.0 and cst.alph[nb, 0] == 1.0
    dz = np.float32(2 * np.float32(0.5 * cs.p_size[2]))  # the +z face offset of the FP32 limiter
    s = _slope_hitting(dz)
    cst.coef[ci, 0, 2, 1:] = [0.0, 0.0, float(s)]
    # a lower y-momentum next door: the face minimum u_min is non-zero
    cst.rhov[ci, 0, 1] = 1e-3
    cst.rhov[nb, 0, 1] = 0.0
    g, o = M.MPM(cs, getattr(abi, "PREC_" + prec_name)), O.Oracle(cs)
    for x in (g, o):
        x.upload_particles(ps)
        x.upload_cells(cst)
        x.upload_lists(off, ent)
        x.Calculate_limiter()
    g.sync()
    lg, lo = g.download_cells().lim_u, o.download_cells().lim_u
    assert np.all(np.isfinite(lo))
    assert np.all(np.isfinite(lg)), np.argwhere(~np.isfinite(lg))[:4]
    assert abs(lg[ci, 0, 2] - lo[ci, 0, 2]) <= 1e-6, (lg[ci, 0, 2], lo[ci, 0, 2])

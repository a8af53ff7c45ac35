"""Host-side pieces of the MGFM seed surrogate: the NumPy restatement used to
check the device kernels (against finite differences), the exact-root targets
(against the oracle's MGFM), the synthetic problem stream and the shipped
weights."""
import numpy as np
import pytest

from tests import mlp_ref as R


def _params(seed=0):
    from pgdg_p2_gb300 import surrogate as S
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(256, R.NI)).astype(np.float32)
    T = rng.normal(size=(256, R.NO)).astype(np.float32)
    return S.init_params(X, T, seed), X, T


def test_layout_matches_library_constants():
    from pgdg_p2_gb300 import surrogate as S
    assert R.NPARAM == S.NPARAM
    assert S.NPARAM + S.NNORM == 9282 + 28


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.1415927, -2.5e-3], np.float32)
    y = R.bf16_round(x)
    assert y[0] == 1.0
    assert y[1] == 1.0            # halfway: ties to even (mantissa ...0)
    assert y[2] == 1.0078125      # rounds up
    assert abs(y[3] - 3.140625) < 1e-7
    assert np.all(np.abs(y - x) <= np.abs(x) * 2.0 ** -8)


def test_numpy_gradient_finite_differences():
    p, X, T = _params(1)
    p = p.astype(np.float64)
    _, g = R.loss_grad(p, X[:64], T[:64])
    rng = np.random.default_rng(2)
    idx = rng.choice(R.NPARAM, 40, replace=False)
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (R.loss_grad(pp, X[:64], T[:64])[0] - R.loss_grad(pm, X[:64], T[:64])[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, fd, g[k])


def test_exact_roots_agree_with_oracle_mgfm(oracle_mod):
    from pgdg_p2_gb300 import surrogate as S
    in6, mat = S.c5_problems(4000, seed=5)
    ps, us, has = S.exact_roots(in6, mat, S.C5_GAMMA, S.C5_PINF)
    res, it = oracle_mod.mgfm_batched(in6, mat, S.C5_GAMMA, S.C5_PINF, 0)
    # the plain Newton solve converges on every problem with a positive root and
    # runs to its cap on nearly all others (a few end within the velocity
    # tolerance while f is still slightly negative)
    assert np.all(it[has] < 50)
    assert np.mean(it[~has] == 50) > 0.99
    tol = np.maximum(1e-8, 1e-3 * np.abs(in6[:, 0] - in6[:, 1]))
    assert np.all(np.abs(res[has, 2] - us[has]) <= tol[has])
    assert np.quantile(np.abs(res[has, 1] - ps[has]) / ps[has], 0.99) < 1e-5


def test_problem_stream_deterministic():
    from pgdg_p2_gb300 import surrogate as S
    a6, am = S.c5_problems(1000, seed=5, offset=500)
    b6, bm = S.c5_problems(1500, seed=5)
    assert np.array_equal(a6, b6[500:]) and np.array_equal(am, bm[500:])
    assert a6[:, 4].min() >= 1e-2 and a6[:, 4].max() <= 1e3
    assert np.abs(a6[:, :2]).max() <= 500
    assert set(np.unique(am)) <= {0, 1, 2, 3}


def test_shipped_weights_are_finite():
    from pgdg_p2_gb300 import surrogate as S
    p = S.load_default()
    if p is None:
        pytest.skip("no trained weights")
    assert p.dtype == np.float32 and p.size == S.NPARAM + S.NNORM
    assert np.all(np.isfinite(p)) and np.all(p[S.NPARAM + S.NI:S.NPARAM + 2 * S.NI] > 0)

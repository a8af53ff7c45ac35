"""Tensor-core (tcgen05) forward pass of the MGFM seed surrogate against the
NumPy restatement with BF16 weights and BF16 activations, and the seeded
batched solve with a tensor-core network."""
import numpy as np
import pytest

from tests import mlp_ref as R
from tests.test_gpu_surrogate import _c5, _check_seeded, _cuda

pytestmark = pytest.mark.gpu


def _forward(gpu_mod, net, X):
    import torch
    Xd = _cuda(X, torch.float32)
    Y = torch.full((len(X), 2), np.nan, dtype=torch.float32, device="cuda:0")
    torch.cuda.synchronize()
    assert gpu_mod.lib().pgdg_surrogate_forward(net.h, Xd.data_ptr(), Y.data_ptr(), len(X)) == 0
    torch.cuda.synchronize()
    return Y.cpu().numpy()


@pytest.mark.parametrize("n", [3000, 128, 1])
def test_tc_forward_matches_bf16_emulation(gpu_mod, n):
    from pgdg_p2_gb300 import surrogate as S
    _, _, X, T, _ = _c5(max(n, 64) * 2, 12)
    X = X[:n]
    for params in (S.init_params(X, T, seed=6), S.load_default()):
        net = S.Surrogate(params, tc=True)
        Y = _forward(gpu_mod, net, X)
        Yr = R.forward_bf16_act(params, X)
        # BF16 activations: the hardware tanh (about 2^-11) can put an activation
        # on the other side of a BF16 rounding boundary than the exact tanh of
        # the emulation, which moves that output by about 1e-2 (typical
        # differences are 1e-7); a wrong operand layout moves outputs by O(1)
        assert np.all(np.isfinite(Y))
        assert np.max(np.abs(Y - Yr)) <= 5e-2, np.max(np.abs(Y - Yr))
        assert np.mean(np.abs(Y - Yr)) <= 1e-3
        net.close()


def test_tc_forward_close_to_cuda_core_forward(gpu_mod):
    from pgdg_p2_gb300 import surrogate as S
    _, _, X, T, _ = _c5(5000, 13)
    p = S.load_default()
    a, b = S.Surrogate(p, tc=True), S.Surrogate(p)
    Ya, Yb = _forward(gpu_mod, a, X), _forward(gpu_mod, b, X)
    # BF16 against FP32 activations through three layers: a few 1e-2 in the
    # normalised output at the 99th percentile (measured 0.037)
    assert np.quantile(np.abs(Ya - Yb)[:, 0], 0.99) <= 0.1
    assert np.mean(np.abs(Ya - Yb)[:, 0]) <= 0.02
    a.close()
    b.close()


def test_tc_seeded_solve(gpu_mod):
    from pgdg_p2_gb300 import surrogate as S
    in6, mat = S.c5_problems(1 << 16, seed=5)
    net = S.Surrogate(S.load_default(), tc=True)
    ip, isd, conv = _check_seeded(in6, mat, S.C5_GAMMA, S.C5_PINF, net)
    assert isd[conv].mean() <= 0.6 * ip[conv].mean()
    net.close()


def test_noalloc_refuses_tc_network(gpu_mod):
    import torch
    from pgdg_p2_gb300 import surrogate as S
    in6, mat = S.c5_problems(64, seed=3)
    net = S.Surrogate(S.load_default(), tc=True)
    t_in, t_m = _cuda(in6, torch.float64), _cuda(mat, torch.int8)
    t_g, t_p = _cuda(S.C5_GAMMA, torch.float64), _cuda(S.C5_PINF, torch.float64)
    out = torch.zeros((64, 3), dtype=torch.float64, device="cuda:0")
    rc = gpu_mod.lib().pgdg_mgfm_batched_noalloc(net.h, t_in.data_ptr(), t_m.data_ptr(), t_g.data_ptr(),
                                                 t_p.data_ptr(), 4, 0, out.data_ptr(), None, 64)
    assert rc == -1
    net.close()

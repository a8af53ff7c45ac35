"""Batched MGFM on the device vs the oracle (FP64, exact operation order)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _run_gpu(M, in6, mat, gam, pinf, variant=0):
    import torch
    dev = torch.device("cuda:0")
    t_in = torch.tensor(in6, dtype=torch.float64, device=dev).contiguous()
    t_m = torch.tensor(mat, dtype=torch.int8, device=dev).contiguous()
    t_g = torch.tensor(gam, dtype=torch.float64, device=dev)
    t_p = torch.tensor(pinf, dtype=torch.float64, device=dev)
    out = torch.zeros((len(in6), 3), dtype=torch.float64, device=dev)
    it = torch.zeros(len(in6), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = M.lib().pgdg_mgfm_batched(None, t_in.data_ptr(), t_m.data_ptr(), t_g.data_ptr(), t_p.data_ptr(), len(gam),
                                   variant, out.data_ptr(), it.data_ptr(), len(in6))
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy(), it.cpu().numpy()


def test_mgfm_known_values(gpu_mod):
    k = json.load(open(os.path.join(HERE, "golden", "mgfm_known.json")))
    out, it = _run_gpu(gpu_mod, np.array(k["in6"]), np.array(k["mat2"]), k["gamma"], k["pinf"])
    assert np.array_equal(out, np.array(k["out3"]))
    assert np.array_equal(it, np.array(k["iters"]))


@pytest.mark.parametrize("variant", [0, 1])
def test_mgfm_bitwise_random(gpu_mod, oracle_mod, variant):
    from tests.golden.make_golden import mgfm_inputs
    rng = np.random.default_rng(11 + variant)
    in6, mat = mgfm_inputs(rng, 1 << 16)
    gam = np.array([1.4, 1.648, 7.15, 2.0])
    pinf = np.array([0.0, 0.0, 3.309e8, 0.0])
    og, ig = _run_gpu(gpu_mod, in6, mat, gam, pinf, variant)
    oo, io = oracle_mod.mgfm_batched(in6, mat, gam, pinf, variant)
    assert np.array_equal(ig, io)
    assert og.tobytes() == oo.tobytes()


@pytest.mark.parametrize("tc", [False, True])
def test_overflowing_seed_falls_back_to_plain(gpu_mod, tc):
    """A network whose output overflows the seed's exponential (here an output
    mean of 1e30) must leave every problem to the plain solve: the same
    results as no network, bit for bit."""
    from pgdg_p2_gb300 import surrogate as S
    from tests.golden.make_golden import mgfm_inputs
    in6, mat = mgfm_inputs(np.random.default_rng(5), 1 << 14)
    gam = np.array([1.4, 1.648, 7.15, 2.0])
    pinf = np.array([0.0, 0.0, 3.309e8, 0.0])
    p = S.baseline_params()
    p[S.NPARAM + 2 * S.NI] = 1e30
    net = S.Surrogate(p, tc=tc)
    out, it = S.mgfm_gpu(in6, mat, gam, pinf, net)
    net.close()
    ref, it_ref = S.mgfm_gpu(in6, mat, gam, pinf, None)
    assert np.all(np.isfinite(out))
    assert out.tobytes() == ref.tobytes()
    assert np.all(it >= it_ref)

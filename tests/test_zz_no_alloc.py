"""pgdg_mgfm_batched_noalloc (seeds in a static device array, no allocation)
against pgdg_mgfm_batched on the same problems, over two consecutive calls.

Both entry points run the same kernels, so the test tolerance is zero: results
and iteration counts must be identical.  Collected last; it passes alone in a
fresh process and after the rest of the suite."""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _noalloc_max():
    hdr = open(os.path.join(os.path.dirname(HERE), "include", "pgdg.h")).read()
    m = re.search(r"#define\s+PGDG_MGFM_NOALLOC_MAX\s+\(1 << (\d+)\)", hdr)
    assert m, "PGDG_MGFM_NOALLOC_MAX not found"
    return 1 << int(m.group(1))


def _device(in6, mat):
    import torch
    from pgdg_p2_gb300 import surrogate as S
    dev = torch.device("cuda:0")
    return (torch.tensor(in6, dtype=torch.float64, device=dev), torch.tensor(mat, dtype=torch.int8, device=dev),
            torch.tensor(S.C5_GAMMA, dtype=torch.float64, device=dev),
            torch.tensor(S.C5_PINF, dtype=torch.float64, device=dev))


def _solve(fn, h, bufs, n):
    import torch
    t_in, t_m, t_g, t_p = bufs
    out = torch.full((n, 3), -7.0, dtype=torch.float64, device="cuda:0")
    it = torch.full((n,), -1, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    rc = fn(h, t_in.data_ptr(), t_m.data_ptr(), t_g.data_ptr(), t_p.data_ptr(), 4, 0, out.data_ptr(), it.data_ptr(), n)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy(), it.cpu().numpy()


@pytest.mark.parametrize("learned", [True, False])
def test_noalloc_matches_allocating_entry_point(gpu_mod, learned):
    from pgdg_p2_gb300 import surrogate as S
    L = gpu_mod.lib()
    net = S.Surrogate(S.load_default()) if learned else None
    h = net.h if net is not None else None
    # two consecutive calls of different sizes; the second is smaller, so a
    # stale seed from the first call would show up if the scratch were misused
    for n, seed in ((200003, 21), (65537, 22)):
        in6, mat = S.c5_problems(n, seed=seed)
        bufs = _device(in6, mat)
        rc_a, out_a, it_a = _solve(L.pgdg_mgfm_batched, h, bufs, n)
        rc_b, out_b, it_b = _solve(L.pgdg_mgfm_batched_noalloc, h, bufs, n)
        assert rc_a == 0 and rc_b == 0
        assert out_b.tobytes() == out_a.tobytes()
        assert np.array_equal(it_b, it_a)
        assert it_b.min() >= 1
    if net is not None:
        net.close()


def test_noalloc_rejects_oversize(gpu_mod):
    from pgdg_p2_gb300 import surrogate as S
    PGDG_EOVERFLOW = -6   # include/pgdg_types.h
    L = gpu_mod.lib()
    net = S.Surrogate(S.load_default())
    in6, mat = S.c5_problems(16, seed=23)
    bufs = _device(in6, mat)
    # the buffers hold 16 problems: an oversize n must be refused before any launch
    rc, out, it = _solve(lambda *a: L.pgdg_mgfm_batched_noalloc(*a[:-1], _noalloc_max() + 1), net.h, bufs, 16)
    assert rc == PGDG_EOVERFLOW
    assert np.all(out == -7.0) and np.all(it == -1)
    net.close()

"""MGFM seed surrogate: data, training and inference helpers.

The network (csrc/k_mlp.cu) predicts, from 12 scale-free features of a
two-material Riemann problem, the star pressure as a log correction to a
closed-form two-shock baseline p_b, scaled by the wave strength
(log(p*/p_b)/sc, sc = s^2/(1+s^2)), and the star velocity (as
(u* - (u_l+u_r)/2)/a0, trained with weight 1/100: it does not seed Newton).  Training targets are exact roots
of the two-shock relation of MPM::MGFM (mpm.cpp:882-926,
glbfunc.h:314-337) found by bisection in FP64; problems without a positive root
(cavitating) are excluded -- the solver sends those straight to the plain solve.

Training data mixes the interface states the solver itself generates (recorded
from the interface queue of the mixed-precision step) with the distribution of
the batched micro-benchmark.  Training runs on the GPU through the library's
own forward/backward/Adam kernels; PyTorch only provides device buffers.
"""
import ctypes as C
import os

import numpy as np

from . import mpm as M

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "mgfm_seed.npy")
NI, NH, NO = 12, 64, 2
NPARAM = NH * NI + NH + NH * NH + NH + NH * NH + NH + NO * NH + NO
NNORM = 2 * NI + 2 * NO
# materials of the micro-benchmark: air, helium, water (stiffened), explosive gas
C5_GAMMA = np.array([1.4, 1.648, 7.15, 2.0])
C5_PINF = np.array([0.0, 0.0, 3.309e8, 0.0])


def _splitmix64(state):
    """Vectorised splitmix64 over an array of uint64 states (returns outputs)."""
    z = (state + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return z ^ (z >> np.uint64(31))


def c5_problems(n, seed=5, offset=0):
    """The batched micro-benchmark's problems: splitmix64(seed) streams; density
    log-uniform on [1e-2, 1e3] per side, pressure ratio log-uniform on [1e-3, 1e4]
    around 1e5 (sides swapped with probability 1/2), normal velocities uniform on
    [-500, 500], material pair uniform over {air, He, water, gas}^2."""
    with np.errstate(over="ignore"):
        idx = np.arange(offset, offset + n, dtype=np.uint64)
        base = (np.uint64(seed) * np.uint64(0x632BE59BD9B4E019) + idx * np.uint64(8)).astype(np.uint64)

        def u(k):
            return (_splitmix64(base + np.uint64(k)) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
        rl = 10 ** (-2 + 5 * u(0))
        rr = 10 ** (-2 + 5 * u(1))
        ratio = 10 ** (-3 + 7 * u(2))
        swap = u(3) < 0.5
        ul = -500 + 1000 * u(4)
        ur = -500 + 1000 * u(5)
        ml = np.minimum((u(6) * 4).astype(np.int64), 3)
        mr = np.minimum((u(7) * 4).astype(np.int64), 3)
    pl = np.full(n, 1e5)
    pr = 1e5 * ratio
    pl2 = np.where(swap, pr, pl)
    pr2 = np.where(swap, pl, pr)
    in6 = np.stack([ul, ur, pl2, pr2, rl, rr], 1)
    mat = np.stack([ml, mr], 1).astype(np.int8)
    return in6, mat


def _W(r, p, ps, g, pinf):
    return np.sqrt(0.5 * r * ((g + 1.0) * ps + (g - 1.0) * p + 2.0 * g * pinf))


def exact_roots(in6, mat, gam, pinf, variant=0):
    """Root p* of f(p) = u_l - u_r - (p-p_l)/W_l - (p-p_r)/W_r (f decreasing) by
    bisection in log p on [1e-8, 1e14], with the MGFM input clamps; returns
    (p*, u*, has_root)."""
    ul, ur, pl, pr, rl, rr = (in6[:, k].astype(np.float64) for k in range(6))
    if variant == 0:
        pl, pr, rl, rr = (np.maximum(x, 1e-10) for x in (pl, pr, rl, rr))
    else:
        pl, pr = np.maximum(pl, 0), np.maximum(pr, 0)
    gl, gr = gam[mat[:, 0]], gam[mat[:, 1]]
    il, ir = pinf[mat[:, 0]], pinf[mat[:, 1]]

    def f(p):
        return ul - ur - (p - pl) / _W(rl, pl, p, gl, il) - (p - pr) / _W(rr, pr, p, gr, ir)
    lo = np.full(len(ul), np.log(1e-8))
    hi = np.full(len(ul), np.log(1e14))
    has = f(np.exp(lo)) >= 0
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        fm = f(np.exp(mid))
        lo = np.where(fm >= 0, mid, lo)
        hi = np.where(fm >= 0, hi, mid)
    ps = np.exp(0.5 * (lo + hi))
    us = ul - (ps - pl) / _W(rl, pl, ps, gl, il)
    return ps, us, has


def baseline_np(ul, ur, pl, pr, rl, rr, gl, il, gr, ir):
    """Closed-form star-pressure baseline of the device (mgfm_baseline): the
    acoustic estimate, then one linearised two-shock step (a pressure, >= 1e-8)."""
    Zl, Zr = np.sqrt(gl * (pl + il) * rl), np.sqrt(gr * (pr + ir) * rr)
    p0 = (Zr * pl + Zl * pr + Zl * Zr * (ul - ur)) / (Zl + Zr)
    p0 = np.where(p0 > 1e-8, p0, 1e-8)
    Wl = np.sqrt(0.5 * rl * ((gl + 1.) * p0 + (gl - 1.) * pl + 2. * gl * il))
    Wr = np.sqrt(0.5 * rr * ((gr + 1.) * p0 + (gr - 1.) * pr + 2. * gr * ir))
    pt = (pl / Wl + pr / Wr + (ul - ur)) / (1. / Wl + 1. / Wr)
    return np.where(pt > 1e-8, pt, 1e-8)


def features_np(in6, mat, gam, pinf):
    """Host restatement of the device feature map (mgfm_features); returns
    (X [n,12] float32, p_b, sc) with the correction scale sc = s^2/(1+s^2)."""
    f32 = np.float32
    ul, ur, pl, pr, rl, rr = (in6[:, k].astype(np.float64) for k in range(6))
    pl, pr, rl, rr = (np.maximum(x, 1e-10) for x in (pl, pr, rl, rr))
    gl, gr = gam[mat[:, 0]], gam[mat[:, 1]]
    il, ir = pinf[mat[:, 0]], pinf[mat[:, 1]]
    Pl, Pr = pl + il, pr + ir
    P0 = np.maximum(Pl, Pr)
    a0 = np.sqrt(P0.astype(f32) / np.sqrt(rl.astype(f32) * rr.astype(f32)))
    du = (ul - ur).astype(f32) / a0
    pb = baseline_np(ul, ur, pl, pr, rl, rr, gl, il, gr, ir)
    lbl = np.log((pb / pl).astype(f32))
    lbr = np.log((pb / pr).astype(f32))
    sv = np.abs(lbl) + np.abs(lbr)
    X = np.stack([np.log((Pl / P0).astype(f32)), np.log((Pr / P0).astype(f32)), np.log((rl / rr).astype(f32)),
                  np.clip(du, f32(-20), f32(20)), lbl, gl.astype(f32), gr.astype(f32), (il / P0).astype(f32),
                  (ir / P0).astype(f32), np.log((pl / P0 + 1e-30).astype(f32)), np.log((pr / P0 + 1e-30).astype(f32)),
                  lbr], 1)
    return X.astype(f32), pb, (sv * sv / (f32(1) + sv * sv)).astype(f32)


def targets_np(in6, mat, gam, pinf, ps, us):
    """Network targets: log(p*/p_b)/sc (0 where sc < 1e-6, clipped to +-6) and
    (u* - (u_l+u_r)/2)/a0."""
    ul, ur = in6[:, 0], in6[:, 1]
    rl, rr = np.maximum(in6[:, 4], 1e-10), np.maximum(in6[:, 5], 1e-10)
    il, ir = pinf[mat[:, 0]], pinf[mat[:, 1]]
    P0 = np.maximum(np.maximum(in6[:, 2], 1e-10) + il, np.maximum(in6[:, 3], 1e-10) + ir)
    a0 = np.sqrt(P0 / np.sqrt(rl * rr))
    _, pb, sc = features_np(in6, mat, gam, pinf)
    sc = sc.astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        y0 = np.where(sc > 1e-6, np.log(ps / pb) / sc, 0.0)
    return np.stack([np.clip(y0, -6, 6), (us - 0.5 * (ul + ur)) / a0], 1).astype(np.float32)


def baseline_params():
    """Parameters whose pressure output is exactly 0: the seed is then the
    closed-form baseline alone (the ablation of the learned correction)."""
    p = np.zeros(NPARAM + NNORM, np.float32)
    p[NPARAM + NI:NPARAM + 2 * NI] = 1.0
    p[NPARAM + 2 * NI + NO:] = 1.0
    return p


class Surrogate:
    """Device-resident MLP: BF16 weights by default (bf16=False: FP32 weights);
    tc=True runs forward passes on the tensor cores with BF16 activations."""

    def __init__(self, params=None, bf16=True, tc=False):
        self.h = C.c_void_p()
        mode = 2 if tc else (1 if bf16 else 0)
        M.check(M.lib().pgdg_surrogate_create(mode, C.byref(self.h)), "pgdg_surrogate_create")
        self.n = M.lib().pgdg_surrogate_num_params()
        assert self.n == NPARAM + NNORM
        if params is not None:
            self.set_params(params)

    def close(self):
        if getattr(self, "h", None):
            M.lib().pgdg_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n
        M.check(M.lib().pgdg_surrogate_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))), "set_params")

    def get_params(self):
        p = np.zeros(self.n, np.float32)
        M.check(M.lib().pgdg_surrogate_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))), "get_params")
        return p


def init_params(Xs, Ts, seed=0):
    """Xavier-initialised weights plus the normalisation statistics of a sample."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM + NNORM, np.float32)
    o = 0
    for fan_out, fan_in in ((NH, NI), (NH, NH), (NH, NH), (NO, NH)):
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        p[o:o + fan_out * fan_in] = rng.uniform(-lim, lim, fan_out * fan_in)
        o += fan_out * fan_in + fan_out
    mx, sx = Xs.mean(0), Xs.std(0) + 1e-6
    my, sy = Ts.mean(0), Ts.std(0) + 1e-6
    sy[1] *= 10.0   # the velocity output does not seed Newton: loss weight 1/100
    p[NPARAM:] = np.concatenate([mx, sx, my, sy]).astype(np.float32)
    return p


def load_default():
    return np.load(WEIGHTS) if os.path.exists(WEIGHTS) else None


def train(Xs, Ts, steps=3000, batch=8192, lr=2e-3, seed=0, log=None, params=None):
    """Train on the GPU with the library's kernels; returns the parameters."""
    import torch
    dev = torch.device("cuda:0")
    net = Surrogate(params if params is not None else init_params(Xs, Ts, seed))
    X = torch.tensor(Xs, device=dev)
    T = torch.tensor(Ts, device=dev)
    n = X.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    loss = C.c_double()
    hist = []
    for it in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).to(dev)
        xb = X[idx].contiguous()
        tb = T[idx].contiguous()
        cur = lr * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * it / steps)))
        torch.cuda.synchronize()
        M.check(M.lib().pgdg_surrogate_train_step(net.h, xb.data_ptr(), tb.data_ptr(), batch, cur, C.byref(loss)),
                "train_step")
        if it % 200 == 0 or it == steps - 1:
            hist.append((it, loss.value))
            if log:
                log(f"step {it} loss {loss.value:.4e}")
    p = net.get_params()
    net.close()
    return p, hist


def mgfm_gpu(in6, mat, gam, pinf, net=None, variant=0):
    """Batched MGFM on the GPU; returns (out3, iterations) on the host."""
    import torch
    dev = torch.device("cuda:0")
    t_in = torch.tensor(np.ascontiguousarray(in6), dtype=torch.float64, device=dev)
    t_m = torch.tensor(np.ascontiguousarray(mat), dtype=torch.int8, device=dev)
    t_g = torch.tensor(gam, dtype=torch.float64, device=dev)
    t_p = torch.tensor(pinf, dtype=torch.float64, device=dev)
    out = torch.zeros((len(in6), 3), dtype=torch.float64, device=dev)
    it = torch.zeros(len(in6), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    M.check(M.lib().pgdg_mgfm_batched(net.h if net is not None else None, t_in.data_ptr(), t_m.data_ptr(),
                                      t_g.data_ptr(), t_p.data_ptr(), len(gam), variant, out.data_ptr(),
                                      it.data_ptr(), len(in6)), "pgdg_mgfm_batched")
    torch.cuda.synchronize()
    return out.cpu().numpy(), it.cpu().numpy()

"""Benchmark of the PGDG per-time-step particle-grid path on GB300.

Metric: cell-stage updates/s = (active cells x 2 RK stages x steps) / time of the
whole step (split, 4x merge, binning, P2G, limiter, DG residual with MGFM,
update, G2P with particle shifting, CFL reduction).  Workload: the 3D Air/He
spherical shock-bubble, 384x96x96 cells, 8 particles per cell (28.3 M
particles), synthetic initial state (seeded lattice), mixed precision.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one per GPU, launched by torch.distributed.run);
the path has no exchange between GPUs.  --impl reference times the CPU
restatement of the reference's path on the host cores (the reference itself
cannot be built: it needs Eigen, oneTBB, Boost.MPI and MPI, none of which are
installed).  One JSON line is printed by rank 0.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell-stage updates/s, learned+mixed vs plain FP64 on GB300 at matched L1 error"
UNIT = "cell-stage/s"
# workloads: config id -> (description, grid, bounded CPU sample grid); the
# default (and the metric's) is the spherical shock-bubble
WORKLOADS = {
    1: ("2D two-phase triple point, 112x48 P1 DG cells, 4 particles/cell", (112, 48, 1), (112, 48, 1)),
    2: ("3D Air/He cylindrical shock-bubble, 256x64x64 P1 DG cells, 8 particles/cell", (256, 64, 64), (64, 16, 16)),
    3: ("3D Air/He spherical shock-bubble, 384x96x96 P1 DG cells, 8 particles/cell", (384, 96, 96), (96, 24, 24)),
    4: ("2D underwater explosion, 1024x1024 P1 DG cells, 4 particles/cell", (1024, 1024, 1), (256, 256, 1)),
}
CONFIG_ID = 3
WORKLOAD, GRID, SAMPLE_GRID = WORKLOADS[CONFIG_ID]


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_value(ms, cells_per_rank, steps):
    """Whole-job cell-stage/s of N independent replicas (one per GPU, no
    exchange between them): all ranks' cell-stages over the slowest rank's time.
    Returns (max ms over ranks, value)."""
    ws, _, _ = _dist()
    if ws > 1:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, ws * cells_per_rank * 2 * steps / (ms / 1e3)


class Clocks:
    """Sample nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_baseline(steps=1, warmup=1, threads=None):
    """The CPU restatement (oracle) timed on a bounded sample of the same case."""
    from oracle import oracle as O
    from pgdg_p2_gb300 import mpm as M
    threads = threads or os.cpu_count()
    O.set_threads(threads)
    cs, p, c = M.make_case(CONFIG_ID, SAMPLE_GRID)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    o.advance(warmup)
    t0 = time.perf_counter()
    o.advance(steps)
    dt = time.perf_counter() - t0
    ncell = cs.ncells
    return {"value": ncell * 2 * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"same case on {SAMPLE_GRID[0]}x{SAMPLE_GRID[1]}x{SAMPLE_GRID[2]} cells "
                      f"({p.n} particles), {steps} step(s) after {warmup} warm-up, FP64 CPU oracle "
                      f"(OpenMP, {threads} threads); reference build unavailable (Eigen/oneTBB/Boost.MPI/MPI absent)",
            "seconds": dt}


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return
    # K steps and W warm-ups of the bounded sample (one sample step takes well
    # under a second on the host cores)
    cb = cpu_baseline(steps=args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * cb["seconds"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_grid": list(SAMPLE_GRID)},
            "cpu_baseline": {"value": cb["value"], "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"],
                             "sample": cb["sample"]},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def pinned_alloc():
    """Array allocator in page-locked host memory (through torch's pinned
    allocator; the arrays keep their buffers alive)."""
    import numpy as np
    import torch

    def alloc(shape, dtype):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        t = torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
        return t.numpy()[:nbytes].view(dtype).reshape(shape)
    return alloc


def state_bytes(p, c):
    tot = 0
    for a in p.as_dict().values():
        tot += a.nbytes
    for a in c.as_dict().values():
        tot += a.nbytes
    return tot


def run_ours(args):
    ws, rank, local = _dist()
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import ctypes
    from pgdg_p2_gb300 import mpm as M
    from pgdg_p2_gb300.abi import PREC_FP64_FMA, PREC_MIXED
    if ws > 1:
        # one replica per GPU: select this rank's device before the context exists
        cudart = ctypes.CDLL("libcudart.so")
        cudart.cudaSetDevice(local)

    from pgdg_p2_gb300 import surrogate as S
    params = S.load_default()
    if params is None:
        raise SystemExit("trained seed weights missing (python -m pgdg_p2_gb300.train_surrogate)")
    net = S.Surrogate(params, tc=True)

    grid = tuple(int(x) for x in args.grid.split(",")) if args.grid else GRID
    cs, p, c = M.make_case(CONFIG_ID, grid)
    ncell = cs.ncells
    g = M.MPM(cs, PREC_MIXED)
    g.set_surrogate(net)
    g.upload_particles(p)
    g.upload_cells(c)
    g.advance(args.warmup)
    g.sync()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: K steps, CUDA events on the context stream ----
    barrier()
    n0 = g.launch_count()
    g.profile(True)
    with Clocks(local) as clk:
        ms = g.time_advance(args.steps)
    prof = g.profile_read()
    g.profile(False)
    launches = g.launch_count() - n0
    barrier()
    ms, value = replica_value(ms, ncell, args.steps)
    st = g.stats()

    if args.only_timed:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
                              "gpu_launches": launches, "stage_ms": {k: v[0] / args.steps for k, v in prof.items()},
                              "tuning": {"pst_variant": g.tune("pst")},
                              "note": "timed region only"}), flush=True)
        g.close()
        return

    # ---- end to end through the C ABI with host buffers in page-locked memory ----
    g2 = M.MPM(cs, PREC_MIXED)
    g2.set_surrogate(net)
    ke = args.steps
    pin = pinned_alloc()
    ph, ch = M.Particles(p.n, cs.dim, alloc=pin), M.Cells(ncell, cs.dim, alloc=pin)
    for k in ph.NAMES:
        getattr(ph, k)[...] = getattr(p, k)
    for k in ch.NAMES:
        getattr(ch, k)[...] = getattr(c, k)
    q = M.Particles(p.n + p.n // 4, cs.dim, alloc=pin)
    cq = M.Cells(ncell, cs.dim, alloc=pin)
    nbytes = state_bytes(ph, ch)
    # warm-up of this context (kernel-variant tuning, first-use buffers), then
    # the timed region starts again from the host state
    g2.upload_particles(ph)
    g2.upload_cells(ch)
    g2.advance(args.warmup)
    g2.sync()
    t0 = time.perf_counter()
    g2.upload_particles(ph)
    g2.upload_cells(ch)
    g2.set_iterate(0)              # the uploaded state is the initial one again
    for _ in range(ke):
        g2.advance(1)
        g2.stats()                 # device->host read of dt / max_v / counters
    g2.download_particles(out=q)
    g2.download_cells(out=cq)
    g2.sync()
    te = time.perf_counter() - t0
    dbytes = (sum(a.nbytes for a in q.as_dict().values()) * q.n // max(q.cap, 1)
              + sum(a.nbytes for a in cq.as_dict().values()))
    e2e = {"value": ws * ncell * 2 * ke / te, "unit": UNIT, "h2d_bytes_per_step": nbytes // ke,
           "d2h_bytes_per_step": dbytes // ke + 160, "steps": ke, "seconds": te}
    g2.close()

    # ---- plain FP64 GPU path (FMA) on the same case, for the mixed/FP64 ratio ----
    f = M.MPM(cs, PREC_FP64_FMA)
    f.upload_particles(p)
    f.upload_cells(c)
    f.advance(1)
    kf = max(1, min(2, args.steps))
    msf = f.time_advance(kf)
    fp64 = {"value": ncell * 2 * kf / (msf / 1e3), "ms_per_step": msf / kf, "steps": kf,
            "speedup_mixed_over_fp64": (ms / args.steps) and (msf / kf) / (ms / args.steps)}
    # matched-error evidence: both paths after the same number of steps from the same state
    nsteps_done = args.warmup + args.steps
    f.advance(nsteps_done - 1 - kf) if nsteps_done - 1 - kf > 0 else None
    import numpy as np
    cg, cf = g.download_cells(), f.download_cells()
    l1 = []
    for u in range(cs.dim + 2):
        qg = (cg.alph * cg.coef[:, :, u, 0]).sum(1)
        qf = (cf.alph * cf.coef[:, :, u, 0]).sum(1)
        l1.append(float(np.abs(qg - qf).sum() / max(np.abs(qf).sum(), 1e-300)))
    mom = sum(float(np.abs((cf.alph * cf.coef[:, :, 1 + k, 0]).sum(1)).sum()) for k in range(cs.dim))
    l1m = [float(np.abs((cg.alph * cg.coef[:, :, 1 + k, 0]).sum(1) - (cf.alph * cf.coef[:, :, 1 + k, 0]).sum(1)).sum()
                 / max(mom, 1e-300)) for k in range(cs.dim)]
    fp64["l1_mixed_vs_fp64"] = {"per_variable": l1, "momentum_over_|rho u|": l1m, "steps": nsteps_done}
    f.close()

    # ---- ablation: mixed path with the reference's inline MGFM and plain seed ----
    a = M.MPM(cs, PREC_MIXED)
    a.upload_particles(p)
    a.upload_cells(c)
    a.advance(args.warmup)
    msa = a.time_advance(kf)
    ablation = {"mixed_inline_plain_seed": {"value": ncell * 2 * kf / (msa / 1e3), "ms_per_step": msa / kf,
                                            "steps": kf}}
    a.close()

    # ---- batched MGFM micro-benchmark (2^24 problems), plain vs learned seed ----
    c5 = None if args.no_c5 else c5_bench(M, S, net)

    # ---- roofline of the dominant kernel ----
    import math
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    # the dominant kernel among those with an algorithmic byte count
    counted = [k for k in prof if k in ("pst", "grid_acc", "g2p", "p2g", "limiter")]
    dom = max(counted, key=lambda k: prof[k][0]) if counted else None
    roof = None
    if dom:
        d_ms, d_cnt = prof[dom]
        per_launch_ms = d_ms / d_cnt
        N = st["n_particles"]
        # algorithmic bytes per launch (FP32 storage) of the dominant kernel
        bytes_per = {"pst": N * (2 * 3 * 4 + 2 * 4 + 4 * 4 + 1 + 1 + 3 * 4 + 3 * 4),
                     "grid_acc": ncell * (2 * 20 * 4 + 2 * 5 * 4 + 2 * 4 + 2 * 20 * 4),
                     "g2p": N * (3 * 4 * 3 + 4 * 9 + 15 * 4 + 3 * 4 * 2) + ncell * 25 * 4,
                     "p2g": ncell * (2 * 4 + 2 * 20 * 4) + N * (3 * 4 + 4 + 1),
                     "limiter": ncell * (2 * 20 * 4 * 1 + 2 * 9 * 4 * 2 + 2 * 5 * 4 + 9 * 4)}.get(dom, 0)
        achieved = bytes_per / (per_launch_ms / 1e3) / 1e9
        # FP32 work of the shifting kernel per particle (3D lattice, 8 per cell): 228
        # candidates x 8 flop (distance test) + 147 members x 33 flop (pair term)
        flops_per = ({"pst": N * (228 * 8 + 147 * 33), "grid_acc": ncell * 13000}.get(dom, 0)
                     if cs.dim == 3 else 0)
        sm_mhz = peaks.get("sm_max_mhz", 2070.0)
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        # DRAM traffic per shifting launch from the ncu capture of the 192x48x48 case
        # (429.4 MB read + written for 3,538,944 particles), scaled by the particle
        # count (the traffic grows with it)
        traffic = 429.4e6 * N / 3538944 if dom == "pst" and CONFIG_ID == 3 else None
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic, "traffic_note": "bytes per launch, ncu capture of "
                "the 192x48x48 case scaled by particles" if traffic else None,
                "peak_source": "measured" if peaks else "fallback",
                "per_launch_ms": per_launch_ms, "launches": d_cnt,
                "fp32": ({"achieved_tflops": flops_per / (per_launch_ms / 1e3) / 1e12,
                          "nominal_peak_tflops": fp32_peak,
                          "frac": flops_per / (per_launch_ms / 1e3) / 1e12 / fp32_peak}
                         if flops_per else None)}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cb = cpu_baseline(steps=1, warmup=1)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "cells": ncell, "particles": st["n_particles"],
                           "precision": "mixed: FP32 DG residual/limiter/G2P/shifting, FP64 MGFM Newton and P2G "
                                        "moment sums", "mgfm_seed": "learned (12-64-64-64-2 MLP, BF16 weights and activations on tcgen05 tensor cores) with plain-Newton fallback; interface problems batched per stage",
                           "l2": "inputs larger than L2 (state of several GB streamed every step)",
                           "parallelism": f"replicas x{ws}"},
                "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof,
                "cpu_baseline": cpu, "fp64_path": fp64, "ablation": ablation, "mgfm_c5": c5,
                "stage_ms": {k: v[0] / args.steps for k, v in prof.items()},
                "tuning": {"pst_variant": g.tune("pst")},
                "stats": {k: st[k] for k in ("n_particles", "n_split", "n_merge", "n_inlet", "n_outlet",
                                             "mgfm_calls", "mgfm_iters", "g2p_fallbacks", "list_entries")}}
        print(json.dumps(line), flush=True)
    g.close()
    net.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def c5_bench(M, S, net, n=1 << 24, reps=3):
    """2^24 seeded two-material problems (splitmix64 seed 5): device time of the
    batched solve from the plain seed and from the learned seed (inputs resident),
    mean/max Newton iterations, and the largest relative p* difference among the
    problems the plain solve converged on."""
    import numpy as np
    import torch
    in6, mat = S.c5_problems(n, seed=5)
    dev = torch.device("cuda:0")
    t_in = torch.tensor(in6, device=dev)
    t_m = torch.tensor(mat, device=dev)
    t_g = torch.tensor(S.C5_GAMMA, device=dev)
    t_p = torch.tensor(S.C5_PINF, device=dev)
    out = {}
    res = {}
    L = M.lib()
    for key, h in (("plain", None), ("learned", net.h)):
        o = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        it = torch.zeros(n, dtype=torch.int32, device=dev)
        args = (h, t_in.data_ptr(), t_m.data_ptr(), t_g.data_ptr(), t_p.data_ptr(), 4, 0, o.data_ptr(),
                it.data_ptr(), n)
        for _ in range(2):
            M.check(L.pgdg_mgfm_batched(*args), "pgdg_mgfm_batched")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.default_stream())
        for _ in range(reps):
            M.check(L.pgdg_mgfm_batched(*args), "pgdg_mgfm_batched")
        e1.record(torch.cuda.default_stream())
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        itn = it.cpu().numpy()
        res[key] = (o.cpu().numpy(), itn)
        out[key] = {"problems_per_s": n / (ms / 1e3), "ms": ms, "mean_iters": float(itn.mean()),
                    "max_iters": int(itn.max())}
    conv = res["plain"][1] < 50
    rel = np.abs(res["learned"][0][conv, 1] - res["plain"][0][conv, 1]) / res["plain"][0][conv, 1]
    out["n"] = n
    out["with_root"] = float(conv.mean())
    out["mean_iters_root"] = {k: float(res[k][1][conv].mean()) for k in res}
    out["max_rel_dp"] = float(rel.max())
    out["speedup_learned_over_plain"] = out["plain"]["ms"] / out["learned"]["ms"]
    return out


def run_c5(args):
    """Config 5 alone: the batched MGFM micro-benchmark (plain vs learned seed)."""
    from pgdg_p2_gb300 import mpm as M
    from pgdg_p2_gb300 import surrogate as S
    net = S.Surrogate(S.load_default(), tc=True)
    c5 = c5_bench(M, S, net, n=args.c5_n)
    print(json.dumps({"metric": "MGFM two-material Riemann problems/s (learned seed, FP64 Newton)",
                      "value": c5["learned"]["problems_per_s"], "unit": "problems/s", "n_gpus": 1,
                      "higher_is_better": True, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": f"{args.c5_n} seeded stiffened-gas interface problems (splitmix64 seed 5)"},
                      "mgfm_c5": c5}), flush=True)
    net.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-c5", action="store_true", help="skip the batched MGFM micro-benchmark")
    ap.add_argument("--only-timed", action="store_true", help="timed region only (profiling runs)")
    ap.add_argument("--grid", default="", help="override the grid, e.g. 192,48,48 (profiling runs)")
    ap.add_argument("--config", type=int, default=3, choices=sorted(WORKLOADS) + [5],
                    help="workload: 1 triple point, 2 cylinder, 3 sphere (default, the metric's), 4 underwater "
                         "explosion, 5 the batched MGFM micro-benchmark alone")
    ap.add_argument("--c5-n", type=int, default=1 << 24, help="problems of the batched MGFM micro-benchmark")
    args = ap.parse_args()
    global CONFIG_ID, WORKLOAD, GRID, SAMPLE_GRID
    if args.config == 5:
        run_c5(args)
        return
    CONFIG_ID = args.config
    WORKLOAD, GRID, SAMPLE_GRID = WORKLOADS[CONFIG_ID]
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

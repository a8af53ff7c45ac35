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
# DRAM bytes read + written per particle by one shifting launch (ncu capture of
# the 192x48x48 sphere: 429.4 MB for 3,538,944 particles)
PST_TRAFFIC_PER_PARTICLE = 429.4e6 / 3538944


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


# through-interaction accuracy runs on the bounded sample grid: steps that take
# each workload well past its first interaction (the C3 sample meets the bubble
# near step 96), and the steps of its bounded CPU-baseline timing
SAMPLE_STEPS = {1: 200, 2: 130, 3: 130, 4: 120}
# simulated time the full-size state is advanced to before the timed steps: the
# shock reaches the bubble at t ~ 0.17 in both 3D shock-bubble cases
REGIME_T = {1: 0.0, 2: 0.2, 3: 0.2, 4: 0.0}


def host_mem_available():
    """Bytes of host memory available (MemAvailable), or None when unknown."""
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except Exception:
        pass
    return None


def oracle_bytes(n_particles, ncells):
    """Host memory of the FP64 oracle holding a case: about 600 B of particle
    state and neighbour lists per particle at 8 per cell, 1.7 kB per cell, and
    the host arrays the case is built in."""
    return int(n_particles * 900 + ncells * 2500)


def run_reference(args):
    """The reference's algorithm on the host cores: the FP64 CPU oracle (the
    reference itself cannot be built here), through its own case builder and
    library only, on the full configuration when the host memory allows."""
    ws, rank, local = _dist()
    if rank != 0:
        return
    from oracle import oracle as O
    threads = os.cpu_count()
    O.set_threads(threads)
    cs = O.case_setup(CONFIG_ID, None)
    grid, note = GRID, ""
    need = oracle_bytes(O.lib().po_case_num_particles(O.C.byref(cs)), cs.ncells)
    avail = host_mem_available()
    if avail is not None and avail < 2 * need:
        grid = SAMPLE_GRID
        note = (f"; host memory available {avail / 2**30:.0f} GiB < 2 x {need / 2**30:.0f} GiB the full case needs, "
                f"so the bounded sample grid ran")
    cs, p, c = O.make_case(CONFIG_ID, grid)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    npart, ncell = p.n, cs.ncells
    del p, c
    o.advance(args.warmup)
    t0 = time.perf_counter()
    o.advance(args.steps)
    dt = time.perf_counter() - t0
    value = ncell * 2 * args.steps / dt
    gl = "x".join(str(x) for x in grid[:cs.dim])
    sample = (f"{'full configuration' if grid == GRID else 'bounded sample'}: {gl} cells ({npart} particles), "
              f"{args.steps} step(s) timed after {args.warmup} warm-up step(s), FP64 CPU oracle (restatement of the "
              f"reference's algorithm; OpenMP, {threads} threads; the reference itself needs Eigen, oneTBB, "
              f"Boost.MPI and MPI, none installed){note}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": list(grid[:cs.dim]), "same_config": grid == GRID},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def accuracy_sample(M, S, net, steps):
    """The learned+mixed path and the plain FP64 GPU path against the FP64
    oracle on the bounded sample grid, through the interaction: relative L1
    per conserved variable (sum |q - q_oracle| / sum |q_oracle| over cells), the
    oracle's own sensitivity to FP32-sized changes of the initial energies (the
    floor a path that stores its state in FP32 meets), and the oracle's host
    time over the same steps (the CPU baseline)."""
    import numpy as np
    from oracle import oracle as O
    from pgdg_p2_gb300.abi import PREC_FP64_FMA, PREC_MIXED
    threads = os.cpu_count()
    O.set_threads(threads)
    cs, p, c = O.make_case(CONFIG_ID, SAMPLE_GRID)
    o, ob = O.Oracle(cs), O.Oracle(cs)
    # the floor: the oracle from energies scaled by 1 +- 2^-24 (seeded signs), the
    # size of rounding the state to FP32
    q = p.copy()
    q.E[:] = q.E * (1.0 + np.random.default_rng(12345).choice([-1.0, 1.0], size=q.E.shape) * 2.0 ** -24)
    o.upload_particles(p)
    ob.upload_particles(q)
    paths = {"mixed_learned": M.MPM(cs, PREC_MIXED), "fp64": M.MPM(cs, PREC_FP64_FMA)}
    paths["mixed_learned"].set_surrogate(net)
    for g in paths.values():
        g.upload_particles(p)
    for x in (o, ob, *paths.values()):
        x.upload_cells(c)
    t_oracle, t_sim = 0.0, 0.0
    for s in range(1, steps + 1):
        t0 = time.perf_counter()
        dt, mv = o.Set_timestep()
        o.set_iterate(s)
        o.MPM_run_simulation(s)
        t_oracle += time.perf_counter() - t0
        t_sim += dt
        for x in (ob, *paths.values()):
            x.Set_timestep()
            x.set_dt(dt)
            x.set_max_v(mv)
            x.set_iterate(s)
            x.MPM_run_simulation(s)

    def l1(cg, co):
        U = cs.dim + 2
        mag = sum(np.abs((co.alph * co.coef[:, :, 1 + k, 0]).sum(1)).sum() for k in range(cs.dim))
        per, mom = [], []
        for u in range(U):
            a = (cg.alph * cg.coef[:, :, u, 0]).sum(1)
            b = (co.alph * co.coef[:, :, u, 0]).sum(1)
            per.append(float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300)))
            if 1 <= u <= cs.dim:
                mom.append(float(np.abs(a - b).sum() / max(mag, 1e-300)))
        return per, mom
    co = o.download_cells()
    floor, floor_m = l1(ob.download_cells(), co)
    so = o.stats()
    out = {"grid": list(SAMPLE_GRID[:cs.dim]), "steps": steps, "t": t_sim,
           "variables": ["rho", "rho u", "rho v", "rho w", "E"] if cs.dim == 3 else ["rho", "rho u", "rho v", "E"],
           "floor_l1": floor, "floor_momentum_over_sum_abs_rho_u": floor_m,
           "oracle": {k: so[k] for k in ("n_split", "n_merge", "n_inlet", "n_outlet", "mgfm_calls", "mgfm_iters")}}
    for name, g in paths.items():
        g.sync()
        per, mom = l1(g.download_cells(), co)
        sg = g.stats()
        out[name] = {"l1": per, "momentum_over_sum_abs_rho_u": mom,
                     "within_1e-3_or_3x_floor": all(e <= max(1e-3, 3 * f) for e, f in zip(per, floor)),
                     "stats": {k: sg[k] for k in ("n_split", "n_merge", "mgfm_calls", "mgfm_iters")}}
        g.close()
    gl = "x".join(str(x) for x in SAMPLE_GRID[:cs.dim])
    cpu = {"value": cs.ncells * 2 * steps / t_oracle, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"same case on {gl} cells ({p.n} particles), the {steps} steps from t = 0 through the "
                     f"shock-bubble interaction (t = {t_sim:.3f}), FP64 CPU oracle (OpenMP, {threads} threads); "
                     f"reference build unavailable (Eigen/oneTBB/Boost.MPI/MPI absent)",
           "seconds": t_oracle}
    return out, cpu


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


def evolve(g, t_end, chunk=25):
    """Untimed set-up: advance the context until its simulated time reaches
    t_end (the state the timed steps start from)."""
    t0 = time.perf_counter()
    n = 0
    while g.stats()["time"] < t_end:
        g.advance(chunk)
        n += chunk
    g.sync()
    return {"t": g.stats()["time"], "steps": n, "seconds": time.perf_counter() - t0}


def totals_drift(a, b):
    """Relative change of the conservation totals between two pgdg_totals reads
    (particle mass per phase, particle energy, cell mass per phase, cell energy)."""
    names = ("particle_mass_1", "particle_mass_2", "particle_energy", "cell_mass_1", "cell_mass_2", "cell_energy")
    return {k: float((b[i] - a[i]) / abs(a[i])) if a[i] != 0 else 0.0 for i, k in enumerate(names)}


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
    del p, c

    # ---- untimed set-up: the state enters the shock-bubble interaction ----
    t_reg = REGIME_T[CONFIG_ID] if args.regime_t < 0 else args.regime_t
    regime = evolve(g, t_reg) if t_reg > 0 else {"t": 0.0, "steps": 0, "seconds": 0.0}
    # the autotuner times the shifting kernel's variants on the state it meets
    # first (t = 0 here); choose again on the interaction state (during warm-up)
    g.tune("pst", -1)
    it_reg = g.stats()["iterate_num"]
    pin = pinned_alloc()
    np_reg = g.num_particles()
    ph = M.Particles(np_reg + np_reg // 4 + 4096, cs.dim, alloc=pin)
    g.download_particles(out=ph)
    ch = g.download_cells(out=M.Cells(ncell, cs.dim, alloc=pin))
    g.advance(args.warmup)
    # and the step graph captured and replayed once (the metric's step loop
    # runs with a warm graph; its capture is setup, like the tuning)
    g.advance(3)
    g.sync()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: K steps as a user runs them (advance: captured step
    # graphs, no per-method events), CUDA events on the context stream ----
    st0, tot0 = g.stats(), g.totals()
    barrier()
    n0 = g.launch_count()
    cu = None
    if args.profile_window:
        cu = ctypes.CDLL("libcuda.so.1")
        cu.cuProfilerStart()
    with Clocks(local) as clk:
        ms = g.time_advance(args.steps)
    if cu is not None:
        cu.cuProfilerStop()
    launches = g.launch_count() - n0
    barrier()
    ms, value = replica_value(ms, ncell, args.steps)
    st, tot1 = g.stats(), g.totals()
    # per-method device times over K further steps (events between the methods,
    # so these steps run eagerly); they explain the timed steps, not replace them
    g.profile(True)
    g.time_advance(args.steps)
    prof = g.profile_read()
    g.profile(False)
    window = {k: st[k] - st0[k] for k in ("n_split", "n_merge", "n_inlet", "n_outlet", "mgfm_calls", "mgfm_iters",
                                           "mgfm_maxit_hits", "g2p_fallbacks")}
    window["mgfm_iters_per_call"] = window["mgfm_iters"] / max(window["mgfm_calls"], 1)
    window["t_start"], window["t_end"] = st0["time"], st["time"]

    if args.only_timed:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
                              "gpu_launches": launches, "stage_ms": {k: v[0] / args.steps for k, v in prof.items()},
                              "tuning": {"pst_variant": g.tune("pst")}, "regime": regime, "window": window,
                              "note": "timed region only"}), flush=True)
        g.close()
        return

    # ---- end to end through the C ABI with host buffers in page-locked memory ----
    # the same regime state, uploaded from the host each time: K x (advance(1) +
    # stats read), then the state is downloaded
    g2 = M.MPM(cs, PREC_MIXED)
    g2.set_surrogate(net)
    ke = args.steps
    q = M.Particles(ph.cap, cs.dim, alloc=pin)
    cq = M.Cells(ncell, cs.dim, alloc=pin)
    nbytes = state_bytes(ph, ch) * ph.n // max(ph.cap, 1)
    # warm-up of this context (kernel-variant tuning, first-use buffers)
    g2.upload_particles(ph)
    g2.upload_cells(ch)
    g2.set_iterate(it_reg)
    g2.advance(args.warmup)
    g2.sync()
    t0 = time.perf_counter()
    g2.upload_particles(ph)
    g2.upload_cells(ch)
    g2.set_iterate(it_reg)
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

    # ---- plain FP64 GPU path (FMA) from the same regime state ----
    f = M.MPM(cs, PREC_FP64_FMA)
    f.upload_particles(ph)
    f.upload_cells(ch)
    f.set_iterate(it_reg)
    f.advance(1)
    kf = max(1, min(2, args.steps))
    f0 = f.stats()
    msf = f.time_advance(kf)
    f1 = f.stats()
    fp64 = {"value": ncell * 2 * kf / (msf / 1e3), "ms_per_step": msf / kf, "steps": kf,
            "speedup_mixed_over_fp64": (msf / kf) / (ms / args.steps),
            "mgfm_iters_per_call": (f1["mgfm_iters"] - f0["mgfm_iters"]) / max(f1["mgfm_calls"] - f0["mgfm_calls"], 1),
            "state": f"the mixed path's state at t = {regime['t']:.3f} (FP32 values promoted)"}
    f.close()

    # ---- ablation from the same regime state: the reference's inline MGFM and plain seed ----
    a = M.MPM(cs, PREC_MIXED)
    a.upload_particles(ph)
    a.upload_cells(ch)
    a.set_iterate(it_reg)
    a.advance(args.warmup)
    a0 = a.stats()
    msa = a.time_advance(kf)
    a1 = a.stats()
    ablation = {"mixed_inline_plain_seed": {
        "value": ncell * 2 * kf / (msa / 1e3), "ms_per_step": msa / kf, "steps": kf,
        "mgfm_iters_per_call": (a1["mgfm_iters"] - a0["mgfm_iters"]) / max(a1["mgfm_calls"] - a0["mgfm_calls"], 1),
        "learned_over_plain": (msa / kf) / (ms / args.steps)}}
    a.close()

    # ---- batched MGFM micro-benchmark (2^24 problems), plain vs learned seed ----
    c5 = None if args.no_c5 else c5_bench(M, S, net)

    # ---- roofline: the shifting kernel and the whole step against the measured FP32 rate ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    with Clocks(local) as clk_peak:
        fp32_plain, _ = M.fp32_peak()
        fp32_packed, _ = M.fp32_peak(packed=True)
    # the FP32 rate is the larger of the single (FFMA) and packed (FFMA2) loops
    fp32_tf = max(fp32_plain, fp32_packed)
    roof = None
    if "pst" in prof:
        d_ms, d_cnt = prof["pst"]
        per_launch_ms = d_ms / d_cnt
        N = st["n_particles"]
        # algorithmic work per shifting launch (3D lattice, 8 per cell): 228 candidate
        # tests x 8 flop and 147 members x 33 flop per particle; bytes: positions at
        # the stage start and end, both smoothing lengths, own density, sound speed,
        # volume and record, phase, mark_in, v in and tv out (74 B)
        flops = N * (228 * 8 + 147 * 33) if cs.dim == 3 else N * (50 * 8 + 32 * 33)
        bytes_per = N * 74
        achieved = flops / (per_launch_ms / 1e3) / 1e12
        # DRAM traffic per shifting launch from the ncu capture of the 192x48x48 case,
        # scaled by the particle count (the traffic grows with it)
        traffic = PST_TRAFFIC_PER_PARTICLE * N if CONFIG_ID == 3 else None
        step_flops = 70000.0 * ncell * 2 if cs.dim == 3 else 11000.0 * ncell * 2
        roof = {"kernel": "pst", "bound": "fp32", "achieved": achieved, "peak": fp32_tf, "unit": "TFLOP/s",
                "frac": achieved / fp32_tf, "traffic": traffic,
                "traffic_note": "bytes per launch: ncu capture of the 192x48x48 case scaled by particles"
                if traffic else None,
                "peak_source": "measured in this run: pgdg_fp32_peak / pgdg_fp32_peak_packed (independent FFMA "
                               "and FFMA2 chains on every SM, CUDA events), the larger; clocks "
                               + json.dumps(clk_peak.summary()),
                "fp32_measured": {"ffma_tflops": fp32_plain, "ffma2_tflops": fp32_packed},
                "per_launch_ms": per_launch_ms, "launches": d_cnt,
                "hbm": {"achieved": bytes_per / (per_launch_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                        "frac": bytes_per / (per_launch_ms / 1e3) / 1e9 / hbm,
                        "peak_source": "measured" if peaks else "fallback"},
                "whole_step": {"achieved": step_flops / (ms / args.steps / 1e3) / 1e12, "peak": fp32_tf,
                               "unit": "TFLOP/s", "frac": step_flops / (ms / args.steps / 1e3) / 1e12 / fp32_tf,
                               "work": "70 kflop per 3D cell-stage (11 kflop in 2D)"}}

    # ---- accuracy through the interaction on the bounded sample, and the CPU baseline ----
    accuracy, cpu = None, None
    if rank == 0 and ws == 1 and not args.no_cpu:
        accuracy, cb = accuracy_sample(M, S, net, SAMPLE_STEPS[CONFIG_ID])
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "cells": ncell, "particles": st["n_particles"],
                           "state": f"advanced untimed to t = {regime['t']:.3f} ({regime['steps']} steps, the "
                                    f"shock-bubble interaction), then {args.warmup} warm-up steps",
                           "precision": "mixed: FP32 DG residual/limiter/G2P/shifting, FP64 MGFM Newton and P2G "
                                        "moment sums",
                           "mgfm_seed": "learned (12-64-64-64-2 MLP, BF16 weights and activations on tcgen05 "
                                        "tensor cores) with plain-Newton fallback; interface problems batched per stage",
                           "l2": "inputs larger than L2 (state of several GB streamed every step)",
                           "graph": "the captured three-step graph warmed by 3 further untimed steps",
                           "parallelism": f"replicas x{ws}"},
                "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof,
                "cpu_baseline": cpu, "fp64_path": fp64, "ablation": ablation, "accuracy": accuracy,
                "window": window, "regime": regime, "conservation": totals_drift(tot0, tot1),
                "mgfm_c5": c5, "stage_ms": {k: v[0] / args.steps for k, v in prof.items()},
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
    # the tail: both seeds meet |f| <= max(1e-8, 1e-3 |u_l - u_r|), which fixes p*
    # only within that band where f is flat; its effect on the ghost state the
    # residual uses (rho*_L and E* = rhoe(p*) + rho* u*^2 / 2 of the left material)
    gam, pinf = S.C5_GAMMA[mat[conv, 0]], S.C5_PINF[mat[conv, 0]]

    def ghost_e(o):
        return (o[:, 1] + gam * pinf) / (gam - 1) + 0.5 * o[:, 0] * o[:, 2] ** 2
    pl, le = res["plain"][0][conv], res["learned"][0][conv]
    rel_rho = np.abs(le[:, 0] - pl[:, 0]) / np.abs(pl[:, 0])
    rel_e = np.abs(ghost_e(le) - ghost_e(pl)) / np.abs(ghost_e(pl))
    out["tail"] = {"problems_rel_dp_above_1e-3": int((rel > 1e-3).sum()),
                   "fraction_rel_dp_above_1e-3": float((rel > 1e-3).mean()),
                   "rel_dp_quantiles": {q: float(np.quantile(rel, float(q))) for q in ("0.5", "0.99", "0.999", "0.9999")},
                   "ghost_rho_max_rel": float(rel_rho.max()), "ghost_rho_rel_q0.999": float(np.quantile(rel_rho, 0.999)),
                   "ghost_E_max_rel": float(rel_e.max()), "ghost_E_rel_q0.999": float(np.quantile(rel_e, 0.999))}
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
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cuProfilerStart/Stop (ncu --profile-from-start off)")
    ap.add_argument("--grid", default="", help="override the grid, e.g. 192,48,48 (profiling runs)")
    ap.add_argument("--config", type=int, default=3, choices=sorted(WORKLOADS) + [5],
                    help="workload: 1 triple point, 2 cylinder, 3 sphere (default, the metric's), 4 underwater "
                         "explosion, 5 the batched MGFM micro-benchmark alone")
    ap.add_argument("--c5-n", type=int, default=1 << 24, help="problems of the batched MGFM micro-benchmark")
    ap.add_argument("--regime-t", type=float, default=-1.0,
                    help="simulated time the state is advanced to (untimed) before the timed steps; -1: the "
                         "workload's default (0.2 for the 3D shock-bubble cases, past the shock-bubble contact)")
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

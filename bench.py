#!/usr/bin/env python
"""Benchmark of the GB300 2PI Kadanoff-Baym step (headline metric: KB steps/s).

Workload (N=1): the Ns=64 lattice, O(N=4), lambda=2, m=1, dt=0.05, memory
window M=1000, tsunami initial state (the large configuration of the
benchmark list). A "step" is one evolve!(t) at a full memory window. The
window is filled by really evolving the first M steps from the initial
state, then W warm-up steps and K timed steps run. The history (2 x 1000^2/2
x 6545 orbits) is far larger than L2, so no flush is needed between steps.

Reported: steps/s of the mixed-precision path (value), the plain FP64 path
on the same workload, their relative difference in n(p,t) and E, the
roofline of the dominant kernel (memory integral), an end-to-end number
through the C ABI with host buffers, GPU clocks during the timed region and
the CPU baseline (the oracle's CPUred port: one warm-up and three timed real
steps at the full window).

--impl reference times the reference's CPU algorithm (the oracle's CPUred
port; the Julia reference cannot run here) on all host cores: W warm-up and
K timed real steps at the full memory window of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "qftdynamicsm.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

CFG = dict(Ns=64, N=4, lam=2.0, mass=1.0, mass2=1.0, dt=0.05, M=1000, init="tsunami")
# smaller case of the same kernels, used for ncu captures (a few GB on the device)
SMALL = dict(Ns=40, N=4, lam=2.0, mass=1.0, mass2=1.0, dt=0.05, M=400, init="tsunami")
METRIC = "KB steps/s at Ns=64 (M=1000 window, mixed precision; plain FP64 GPU alongside)"


def metric_name():
    """The headline metric; other lattices or windows (sweeps, profiler cases) name theirs."""
    if (CFG["Ns"], CFG["M"]) == (64, 1000):
        return METRIC
    return f"KB steps/s at Ns={CFG['Ns']} (M={CFG['M']} window, mixed precision)"


def workload_name():
    return (f"KB step at full memory window: Ns={CFG['Ns']}, N={CFG['N']}, lambda={CFG['lam']:g}, "
            f"m={CFG['mass']:g}, dt={CFG['dt']:g}, M={CFG['M']}, tsunami initial state")


def num_orbits(Ns):
    """Cubic orbits of an Ns^3 lattice: C(Ns/2 + 3, 3)."""
    return math.comb(Ns // 2 + 3, 3)


def bench_config(ws):
    """The workload as both arms name it (identical dicts; precision is in dtype)."""
    return {"workload": workload_name() + ", LambdaNLO", "orbits": num_orbits(CFG["Ns"]),
            "l2": "no flush: the two-time history (GBs) is >> 129 MB L2",
            "parallelism": "replicas" if ws > 1 else "single"}


def tsunami_n(k2):
    return 5.0 * np.exp(-((np.sqrt(k2) - 1.0) ** 2) / (2 * 0.2 ** 2))


def gap_mass(k2, deg, n, lam, N, mass2, vol):
    from kb2pi.twopiscalar import Discretization, Phi4, getGapMass

    disc = Discretization(1.0, CFG["Ns"], 3, 0, CFG["dt"], vol, 1.0 / vol, CFG["M"], 0)
    return getGapMass(Phi4(lam, N, mass2), "LambdaNLO", disc, n, k2, deg)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", self.gpu], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("KB_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_handle(precision, device):
    from kb2pi import capi

    p = capi.KbParams(Ns=CFG["Ns"], sdim=3, M=CFG["M"], N=CFG["N"], pexp=1, precision=precision, device=device,
                      flags=0, dt=CFG["dt"], lam=CFG["lam"], mass2=CFG["mass2"], mass=CFG["mass"])
    return capi.Handle([p])


def apply_tuning(h, args, fp64=False):
    """Autotune the launch configuration on the filled window (untimed), unless fixed on the command line."""
    if any(v is not None for v in (args.memint_variant, args.sunset_grid, args.batch_order, args.sunset_variant,
                                   args.memint_split, args.batch_overlap, args.memint_persistent)):
        h.set_tuning(memint_variant=None if fp64 else args.memint_variant, sunset_grid=args.sunset_grid,
                     batch_order=args.batch_order, sunset_variant=None if fp64 else args.sunset_variant,
                     memint_split=args.memint_split, batch_overlap=args.batch_overlap,
                     memint_persistent=args.memint_persistent)
        d = h.tuning()
        d["source"] = "command line"
        return d
    d = h.autotune(trials=3)
    d["source"] = "kb_autotune"
    return d


def init_and_fill(h):
    _, k2, deg = h.orbits(0)
    n = tsunami_n(k2)
    m0 = gap_mass(k2, deg, n, CFG["lam"], CFG["N"], CFG["mass2"], CFG["Ns"] ** 3)
    h.init(0, n, m0)
    # evolve until the memory window is full (t = M), measuring once at the end
    h.steps(3, CFG["M"] - 2, 0)
    return CFG["M"]


def sample_rows(h, t):
    """F(t, t') and rho(t, t') of run 0 at a few t' across the window (host copies)."""
    tmin, _ = h.window(0)
    tps = [tp for tp in (t, t - 1, t - 10, t - 100, t - 500, tmin) if tp >= tmin]
    return [np.array([h.get(0, w, t, tp) for tp in tps]) for w in (0, 1)]


def rows_rel_err(a, b):
    """max over rows of max|a - b| / max|b| (rows whose reference is zero, rho(t,t), skipped)."""
    worst = 0.0
    for x, y in zip(a, b):
        m = float(np.max(np.abs(y)))
        if m > 0.0:
            worst = max(worst, float(np.max(np.abs(x - y))) / m)
    return worst


def timed_steps(h, t0, K, stream_ptr):
    import torch

    st = torch.cuda.ExternalStream(stream_ptr)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    h.sync()
    torch.cuda.synchronize()
    e0.record(st)
    for i in range(K):
        h.step(t0 + i)
    e1.record(st)
    e1.synchronize()
    h.sync()
    return e0.elapsed_time(e1)


def timed_graph_steps(h, t0, K, stream_ptr):
    import torch

    st = torch.cuda.ExternalStream(stream_ptr)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    h.sync()
    e0.record(st)
    h.steps(t0, K, 0)
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sunset_flops(Ns, S, rows):
    """Useful FP32 flops of the sunset per step: per t' row, four orbit cosine
    transforms of 2 H^2 P + S H multiply-adds each (H = Ns/2+1, P = H(H+1)/2)."""
    H = Ns // 2 + 1
    P = H * (H + 1) // 2
    return 2.0 * 4 * (2 * H * H * P + S * H) * rows


def fp32_fma_peak_tflops(device):
    """Nominal FP32 FMA rate: SMs x 128 lanes x 2 flops x maximum SM clock."""
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    except Exception:
        pass
    try:
        import torch

        nsm = torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        nsm = 152
    return nsm * 128 * 2 * mhz * 1e6 / 1e12


def read_traffic(key):
    """Per-launch DRAM bytes of the memory-integral kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "memint_mixed_ns64_m1000.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def algorithmic_bytes(M, S, b_hist, b_sig):
    """Unique bytes of one memory-integral launch: the two-time triangle of F and rho
    read once, the new row written, the self-energy row read."""
    return 2 * (M * (M + 1) // 2) * S * b_hist + 2 * M * S * b_hist + 2 * M * S * b_sig


# ---------------------------------------------------------------------------
def host_mem_available():
    """MemAvailable of the host in bytes (None where /proc/meminfo is absent)."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def cpu_window():
    """Memory window of the CPU runs: the workload's M when its FP64 orbit history
    (2 x M(M+1)/2 x S doubles, the reference's CPUred storage) fits in 80 % of the
    host's available memory, else the largest M that does."""
    M, S = CFG["M"], num_orbits(CFG["Ns"])
    avail = host_mem_available()
    if avail is None:
        return M
    while M > 8 and 2 * (M * (M + 1) // 2) * S * 8 > 0.8 * avail:
        M -= 8
    return M


def cpu_baseline(steps, warmup, budget_s=None, window=None):
    """The oracle's CPUred port (ENGINE_ORBIT: orbit history, full-lattice rfft/brfft
    sunset, memory integrals that read each history slot twice) on all host cores,
    timed over real KB steps at a full memory window. The window is filled by
    expandSimData! alone, as the reference benchmark does (TwoPIScalar_Bechmark.jl:62-104),
    then `warmup` untimed and up to `steps` timed evolve! steps run; the timed loop
    stops early (after at least min(steps, 3) steps) once budget_s seconds are spent.
    Returns the cpu_baseline object; 'steps_timed' is the number of steps timed."""
    from oracle import ENGINE_ORBIT, Oracle

    threads = os.cpu_count() or 1
    M = window or cpu_window()
    o = Oracle(CFG["Ns"], 3, M=M, N=CFG["N"], dt=CFG["dt"], lam=CFG["lam"], mass2=CFG["mass2"],
               mass=CFG["mass"], engine=ENGINE_ORBIT, nthreads=threads)
    try:
        _, k2, deg = o.orbits()
        o.init_occupation(tsunami_n(k2), 1.0)
        for _ in range(3, M + 1):
            o.expand()
        t = M
        for _ in range(warmup):
            t += 1
            o.step(t)
        ts, sun, rest = [], [], []
        t_start = time.perf_counter()
        kmin = min(steps, 3)
        for _ in range(steps):
            if len(ts) >= kmin and budget_s is not None and time.perf_counter() - t_start > budget_s:
                break
            t += 1
            a = time.perf_counter()
            o.step(t)
            ts.append(time.perf_counter() - a)
            s_sun, s_rest = o.step_times()
            sun.append(s_sun)
            rest.append(s_rest)
    finally:
        o.close()
    total = sum(ts)
    return {"value": len(ts) / total, "unit": "steps/s", "cores": threads, "kind": "port",
            "steps_timed": len(ts), "s_per_step": total / len(ts),
            "s_sunset_per_step": sum(sun) / len(ts), "s_rest_per_step": sum(rest) / len(ts),
            "sample": f"oracle CPUred port (orbit history, full-lattice rfft/brfft sunset, memory integrals "
                      f"reading each slot twice), Ns={CFG['Ns']}, M={M} window filled by expand, {warmup} "
                      f"warm-up + {len(ts)} timed full-window steps, {threads} threads"
                      + ("" if M == CFG["M"] else
                         f"; window M={M} instead of the workload's M={CFG['M']} "
                         + ("(command line)" if window else "(to fit host memory)"))}


def measure_batched(local, seed, steps, warmup, args=None, ws=1):
    """Config 3 on one device: 64 independent runs with uneven Ns, lambda, T and memory
    windows in one launch per kernel (mixed precision, graph-captured steps), 500 steps each.
    Returns run-steps/s and its parts."""
    from kb2pi import capi

    rng = np.random.default_rng(seed)
    runs = []
    for r in range(64):
        runs.append(dict(Ns=int(rng.choice([16, 24, 32, 48])), lam=float(rng.uniform(0.5, 8.0)),
                         T=float(rng.uniform(0.5, 3.0)), M=int(rng.integers(100, 501))))
    ps = [capi.KbParams(Ns=c["Ns"], sdim=3, M=c["M"], N=4, pexp=1, precision=capi.KB_PREC_MIXED, device=local,
                        flags=0, dt=0.05, lam=c["lam"], mass2=1.0, mass=1.0) for c in runs]
    h = capi.Handle(ps)
    for r, c in enumerate(runs):
        _, k2, _ = h.orbits(r)
        n = 1.0 / (np.exp(np.sqrt(k2 + 1.0) / c["T"]) - 1.0)
        h.init(r, n, 1.0)
    # 500 steps each: the first 500 - K - W fill every memory window, W warm up, K are timed
    total = 500
    fill = max(0, total - steps - warmup)
    h.steps(3, fill, 0)
    t = 2 + fill
    h.steps(t + 1, warmup, 0)
    t += warmup
    if args is not None:
        tuning = apply_tuning(h, args)
    else:
        tuning = h.autotune(trials=3)
        tuning["source"] = "kb_autotune"
    stream = h.stream()
    barrier(ws)
    with ClockSampler(local) as clk:
        ms = timed_graph_steps(h, t + 1, steps, stream)
    t += steps
    ms = max_over_ranks(ws, ms)
    # per-kernel times of a few more steps (events around each launch)
    h.profile(True)
    for i in range(3):
        h.step(t + 1 + i)
    prof = h.profile_read()
    h.profile(False)
    h.close()
    return {"value": ws * 64 * steps / (ms / 1000.0), "ms_per_step": ms / steps, "runs": runs, "tuning": tuning,
            "clocks": clk.summary(),
            "kernels_ms": {"memint": prof["memint"][0] / max(1, prof["memint"][1]),
                           "sunset": prof["sunset"][0] / max(1, prof["sunset"][1])}}


def run_batched(args):
    """Config 3: 64 independent runs with uneven Ns, lambda, T and memory windows in one
    launch per kernel (mixed precision, graph-captured steps). Reports run-steps/s."""
    import torch

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    b = measure_batched(local, args.seed, args.steps, args.warmup, args, ws)
    if rank != 0:
        return 0
    tuning = b["tuning"]
    line = {"metric": "run-steps/s, 64 uneven runs in one launch (config 3)", "value": b["value"],
            "unit": "run-steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 history/sunset, f64 accumulation/leapfrog/diagnostics",
            "data": f"synthetic: thermal states, per-run draws seeded with {args.seed}",
            "config": {"workload": "64 runs, Ns in {16,24,32,48}, lambda U[0.5,8], T U[0.5,3], M U{100..500}, "
                                   "dt=0.05, steps 478..500 of 500", "runs": b["runs"]},
            # per graph step: advance_t_kernel, then per group (one, or two with batch_overlap) the
            # sunset and memint kernels (+ memint_finish_kernel when split)
            "clocks": b["clocks"],
            "gpu_launches": (1 + (2 if tuning.get("batch_overlap") else 1) * (2 + bool(tuning.get("memint_split"))))
            * args.steps,
            "tuning": tuning,
            "kernels_ms": b["kernels_ms"]}
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint(args):
    """Config 4: gradient of the shell-averaged late-time occupation (8 radial
    shells) plus the total energy at Ns=24, window 300, 300 steps, with respect
    to lambda, m^2 and 8 Gaussian-bump amplitudes of the initial occupation;
    checkpoint every 20 steps, FP64. Reports gradients/s of kb_adjoint and the
    agreement with central finite differences of the GPU forward run."""
    import torch

    from kb2pi import adjoint as adj
    from kb2pi import capi

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    cfg = dict(Ns=24, N=4, lam=2.0, mass2=1.0, mass=1.0, dt=0.05, M=300, pexp=1, device=local)
    tf, ckpt, nb = 302, 20, 8
    h = capi.Handle([adj.params_for(cfg, 0)])
    _, k2, deg = h.orbits()
    h.close()
    rng = np.random.default_rng(args.seed)
    amps = rng.uniform(0.0, 5.0, nb)
    B = adj.bump_basis(k2, nb)
    wn = adj.shell_weights(k2, deg, nb)
    n0 = amps @ B

    def fwd(c, n):
        hh = capi.Handle([adj.params_for(c, 0)])
        hh.init(0, n, 1.0)
        hh.steps(3, tf - 2, 0)
        m = hh.measure(0, tf)
        hh.close()
        return float(np.dot(wn, m["n"]) + m["E"])

    r = adj.loss_and_grad(cfg, n0, tf, w_n=wn, w_E=1.0, ckpt_every=ckpt)  # warm-up
    K = max(1, min(args.steps, 3))
    barrier(ws)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(K):
            r = adj.loss_and_grad(cfg, n0, tf, w_n=wn, w_E=1.0, ckpt_every=ckpt)
        torch.cuda.synchronize()
        dt_adj = (time.perf_counter() - t0) / K
    t0 = time.perf_counter()
    L = fwd(cfg, n0)
    dt_fwd = time.perf_counter() - t0
    dt_adj = max_over_ranks(ws, dt_adj)
    if rank != 0:
        return 0
    # central finite differences (step 1e-5 relative) of the GPU forward run
    def cd(f, x):
        e = 1e-5 * max(abs(x), 1.0)
        return (f(x + e) - f(x - e)) / (2 * e)
    fd = {"lambda": cd(lambda v: fwd(dict(cfg, lam=v), n0), cfg["lam"]),
          "mass2": cd(lambda v: fwd(dict(cfg, mass2=v), n0), cfg["mass2"])}
    ga = B @ r["n_init"]
    fd_a = np.array([cd(lambda s, b=b: fwd(cfg, (amps + s * np.eye(nb)[b]) @ B), 0.0) for b in range(nb)])
    errs = {"lambda": abs(r["lambda"] - fd["lambda"]) / abs(fd["lambda"]),
            "mass2": abs(r["mass2"] - fd["mass2"]) / abs(fd["mass2"]),
            "amplitudes": float(np.max(np.abs(ga - fd_a)) / np.max(np.abs(fd_a)))}
    line = {"metric": "adjoint gradients/s (config 4: Ns=24, window 300, 300 steps, checkpoint every 20)",
            "value": ws / dt_adj, "unit": "gradients/s", "n_gpus": ws, "steps": K, "warmup": 1,
            "ms_per_step": 1000.0 * dt_adj, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": f"synthetic: 8 bump amplitudes U[0,5] seeded with {args.seed}",
            "config": {"workload": "loss = sum over 8 radial shells of the mean n(p, t=302) + E(302); "
                                   "Ns=24, N=4, lambda=2, m^2=1, dt=0.05, M=300, 300 steps, ckpt_every=20"},
            "loss": r["loss"], "loss_forward": L, "forward_s": dt_fwd,
            "grad": {"lambda": r["lambda"], "mass2": r["mass2"], "amplitudes": ga.tolist()},
            "fd": {"lambda": fd["lambda"], "mass2": fd["mass2"], "amplitudes": fd_a.tolist()},
            "rel_err_vs_fd": errs, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_ninverse(args):
    """1/N expansion at NLO (NinverseNLO), FP64: Ns=32, N=4, lambda=4, dt=0.05, M=400,
    tsunami state; steps/s at a full window, the self-energy share (bubbles, Volterra
    solves, Sigma) and the memory integrals timed with events."""
    import torch

    from kb2pi import capi

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    Ns, M = args.ns or 32, args.m or 400
    p = capi.KbParams(Ns=Ns, sdim=3, M=M, N=4, pexp=capi.KB_PEXP_NINV_NLO, precision=capi.KB_PREC_FP64,
                      device=local, flags=0, dt=0.05, lam=4.0, mass2=1.0, mass=1.0)
    h = capi.Handle([p])
    _, k2, deg = h.orbits(0)
    n = tsunami_n(k2)
    h.init(0, n, gap_mass(k2, deg, n, 4.0, 4, 1.0, Ns ** 3))
    h.steps(3, M - 2, 0)
    t = M
    h.steps(t + 1, args.warmup, 0)
    t += args.warmup
    tuning = apply_tuning(h, args, fp64=True)
    stream = h.stream()
    barrier(ws)
    h.profile(True)
    with ClockSampler(local) as clk:
        ms = timed_steps(h, t + 1, args.steps, stream)
    prof = h.profile_read()
    h.profile(False)
    m = h.measure(0, t + args.steps)
    h.close()
    ms = max_over_ranks(ws, ms)
    if rank != 0:
        return 0
    line = {"metric": "KB steps/s, 1/N expansion at NLO (NinverseNLO), FP64", "value": ws * args.steps / (ms / 1e3),
            "unit": "steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic: tsunami initial state, gap-mass init",
            "config": {"workload": f"NinverseNLO, Ns={Ns}, N=4, lambda=4, dt=0.05, M={M}, full window"},
            "kernels_ms": {"self_energies": prof["sunset"][0] / max(1, prof["sunset"][1]),
                           "memint": prof["memint"][0] / max(1, prof["memint"][1])},
            # per step: set_t_kernel, the three 1/N kernels, memint_kernel (+ memint_finish_kernel when split)
            "E": m["E"], "tuning": tuning, "clocks": clk.summary(),
            "gpu_launches": (5 + bool(tuning.get("memint_split"))) * args.steps}
    print(json.dumps(line), flush=True)
    return 0

def run_reference(args):
    """The reference's algorithm on the host cores: the oracle's CPUred port at the
    benchmark workload, W warm-up and K timed real steps at a full window (fewer timed
    steps, at least three, if they would run past about four minutes)."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    cb = cpu_baseline(steps=max(1, args.steps), warmup=args.warmup, budget_s=240.0, window=args.cpu_window)
    k = cb["steps_timed"]
    line = {"impl": "reference", "metric": metric_name(), "value": cb["value"], "unit": "steps/s", "n_gpus": args.gpus,
            "steps": k, "warmup": args.warmup, "ms_per_step": 1000.0 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: tsunami initial state n(p)=5exp(-(|p|-1)^2/0.08), window filled by expand",
            "config": bench_config(args.gpus),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = local
    from kb2pi import capi

    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    phys = int(cvd.split(",")[local]) if cvd and cvd.split(",")[local].isdigit() else local

    # --- mixed precision (headline) ------------------------------------------------
    h = make_handle(capi.KB_PREC_MIXED, dev)
    S = h.S[0]
    t = init_and_fill(h)
    meas_mixed = h.measure(0, t)
    rows_mixed = sample_rows(h, t)
    tuning = apply_tuning(h, args)
    for i in range(args.warmup):
        h.step(t + 1 + i)
    t += args.warmup
    stream = h.stream()
    barrier(ws)
    h.profile(True)
    with ClockSampler(phys) as clk:
        ms = timed_steps(h, t + 1, args.steps, stream)
    t += args.steps
    prof = h.profile_read()
    h.profile(False)
    ms = max_over_ranks(ws, ms)
    barrier(ws)
    ms_per_step = ms / args.steps
    value = ws * args.steps / (ms / 1000.0)

    # graph-captured steps (same work, one graph launch per step)
    gms = timed_graph_steps(h, t + 1, args.steps, stream)
    t += args.steps

    # end to end through the C ABI with host buffers: per step kb_step (t by value)
    # and the step's measurement (scalars + per-orbit arrays) back to the host,
    # read one step behind (kb_measure_enqueue / kb_measure_take) so that the
    # device runs step t+1 while the host takes step t
    h.sync()
    n_host = np.zeros(S)
    t0 = time.perf_counter()
    h.step(t + 1)
    h.measure_enqueue(0, t + 1)
    for i in range(args.steps):
        if i + 1 < args.steps:
            h.step(t + 2 + i)
            h.measure_enqueue(0, t + 2 + i)
        m = h.measure_take(0, t + 1 + i)
        n_host[:] = m["n"]
    e2e_s = time.perf_counter() - t0
    t += args.steps
    e2e_s = max_over_ranks(ws, e2e_s)
    e2e_val = ws * args.steps / e2e_s
    d2h = 5 * S * 8 + (4 * ((S + 7) // 8)) * 8  # per-orbit arrays + energy partials

    # the same steps with Kahan-compensated FP32 tile sums in the memory integrals
    comp = None
    if tuning.get("memint_variant") == 2:
        h.set_tuning(memint_compensated=1)
        for i in range(2):
            h.step(t + 1 + i)
        t += 2
        cms = timed_steps(h, t + 1, args.steps, stream)
        t += args.steps
        h.set_tuning(memint_compensated=0)
        comp = {"steps_per_s": args.steps / (cms / 1000.0), "ms_per_step": cms / args.steps,
                "what": "memint_compensated = 1 (Kahan sums of the FP32 tile partials), same tuning otherwise"}
    h.close()
    del h

    # --- plain FP64 path on the same workload ----------------------------------------
    fp64 = None
    if not args.no_fp64:
        h64 = make_handle(capi.KB_PREC_FP64, dev)
        t64 = init_and_fill(h64)
        meas64 = h64.measure(0, t64)
        rows64 = sample_rows(h64, t64)
        tuning64 = apply_tuning(h64, args, fp64=True)
        for i in range(min(args.warmup, 3)):
            h64.step(t64 + 1 + i)
        t64 += min(args.warmup, 3)
        k64 = max(3, min(args.steps, args.fp64_steps))
        h64.profile(True)
        ms64 = timed_steps(h64, t64 + 1, k64, h64.stream())
        prof64 = h64.profile_read()
        h64.close()
        ms64 = max_over_ranks(ws, ms64)
        nn = meas64["n"]
        fp64 = {"steps_per_s": ws * k64 / (ms64 / 1000.0), "ms_per_step": ms64 / k64, "steps": k64,
                "tuning": tuning64,
                "memint_ms": prof64["memint"][0] / max(1, prof64["memint"][1]),
                "sunset_ms": prof64["sunset"][0] / max(1, prof64["sunset"][1]),
                "mixed_vs_fp64_rel_err": {
                    "n": float(np.max(np.abs(meas_mixed["n"] - nn)) / np.max(np.abs(nn))),
                    "E": abs(meas_mixed["E"] - meas64["E"]) / abs(meas64["E"]),
                    "F": rows_rel_err(rows_mixed[0], rows64[0]), "rho": rows_rel_err(rows_mixed[1], rows64[1]),
                    "at_t": t64 - min(args.warmup, 3),
                    "rows": "F(t,t'), rho(t,t') at t' = t, t-1, t-10, t-100, t-500, tmin; each row's error "
                            "normalised by its max"}}

    if rank != 0:
        return 0
    M = CFG["M"]
    mi_ms = prof["memint"][0] / max(1, prof["memint"][1])
    sun_ms = prof["sunset"][0] / max(1, prof["sunset"][1])
    alg = algorithmic_bytes(M, S, 4, 4)
    peak, peak_kind = read_peaks()
    achieved = alg / (mi_ms / 1000.0) / 1e9
    # the committed capture covers this workload only
    # memory-integral kernels of the chosen configuration; the committed capture
    # the batched form (config 3) in the same run, autotuned, 10 timed graph steps
    batched = None
    if ws == 1 and not args.no_batched and args.config == "c5" and not (args.ns or args.m):
        try:
            b = measure_batched(dev, args.seed, 10, 3)
            batched = {"metric": "run-steps/s, 64 uneven runs in one launch (config 3)", "value": b["value"],
                       "unit": "run-steps/s", "ms_per_step": b["ms_per_step"], "steps": 10, "warmup": 3,
                       "tuning": b["tuning"], "kernels_ms": b["kernels_ms"], "clocks": b["clocks"],
                       "workload": "64 runs drawn with seed %d: Ns in {16,24,32,48}, lambda U[0.5,8], T U[0.5,3], "
                                   "M U{100..500}, dt=0.05, steps 488..500 of 500" % args.seed}
        except Exception as e:  # reported beside the headline, not required for it
            batched = {"value": None, "error": str(e)}

    # covers the benchmark workload in each mode
    split = bool(tuning.get("memint_split"))
    if tuning.get("memint_variant") == 0:
        mi_kernel, key = "memint_blk_kernel<3>", None
    elif tuning.get("memint_variant") == 2 and tuning.get("memint_split") == 2:
        mi_kernel, key = ("memint_kernel<float,32,3,2,split,leapfrog warps> (whole waves whole, the rest split) + "
                          "memint_finish_kernel", "traffic_bytes_per_step_tail_lfw")
    elif tuning.get("memint_variant") == 2:
        mi_kernel, key = "memint_kernel<float,32,3,2,whole,leapfrog warps>", "traffic_bytes_per_launch_lfw"
    elif tuning.get("memint_split") == 2:
        mi_kernel, key = ("memint_kernel<float,32,3,2,split> (whole waves whole, the rest split) + "
                          "memint_finish_kernel", "traffic_bytes_per_step_tail")
    elif split:
        mi_kernel, key = "memint_kernel<float,32,3,2,split> + memint_finish_kernel", "traffic_bytes_per_step_split"
    else:
        mi_kernel, key = "memint_kernel<float,32,3,2>", "traffic_bytes_per_launch"
    if tuning.get("memint_persistent"):
        mi_kernel += " (persistent grid, one CTA per SM)"
    # the committed full-size capture covers the persistent tail-split form only
    if key != "traffic_bytes_per_step_tail_lfw" or not tuning.get("memint_persistent"):
        key = None
    traffic = read_traffic(key) if key and (CFG["Ns"], CFG["M"]) == (64, 1000) else None
    fp32_peak = fp32_fma_peak_tflops(local)
    line = {
        "metric": metric_name(), "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 history/sunset, f64 accumulation/leapfrog/diagnostics",
        "data": "synthetic: tsunami initial state n(p)=5exp(-(|p|-1)^2/0.08), window filled by real evolution",
        "config": bench_config(ws),
        "history_GB": 2 * ((S + 7) // 8) * 8 * ((M + 31) // 32 * 32) ** 2 * 4 / 1e9,
        "mode_steps_per_s": value * M * CFG["Ns"] ** 3,
        "graph_ms_per_step": gms / args.steps,
        "kernels_ms": {"memint": mi_ms, "sunset": sun_ms},
        "tuning": tuning,
        "sunset": {"bound": "FP32 CUDA cores (shared-memory operand traffic and barriers between passes); "
                            "flops counted as the direct cosine transforms (passes 1 and 3 run folded)",
                   "useful_gflop_per_step": sunset_flops(CFG["Ns"], S, M - 1) / 1e9,
                   "achieved_tflops": sunset_flops(CFG["Ns"], S, M - 1) / (sun_ms / 1000.0) / 1e12,
                   "fp32_fma_peak_tflops": fp32_peak,
                   "frac": sunset_flops(CFG["Ns"], S, M - 1) / (sun_ms / 1000.0) / 1e12 / fp32_peak,
                   "peak_kind": "nominal (SMs x 128 x 2 x max SM clock)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": mi_kernel, "algorithmic_bytes": alg},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_val, "unit": "steps/s", "h2d_bytes_per_step": 4, "d2h_bytes_per_step": d2h,
                "path": "kb_step + kb_measure_enqueue/kb_measure_take (one step behind) through the C ABI, "
                        "host buffers, wall clock"},
        # per timed step: set_t_kernel, sunset_kernel, memint_kernel (+ memint_finish_kernel when split)
        "gpu_launches": (4 if split else 3) * args.steps,
        "fp64_plain": fp64,
        "compensated_sums": comp,
        "speedup_mixed_vs_fp64": (value / fp64["steps_per_s"]) if fp64 else None,
        "batched_64_runs": batched,
    }
    if ws == 1 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_baseline(steps=3, warmup=1, budget_s=30.0, window=args.cpu_window)
        except Exception as e:  # the baseline is reported, not required
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--cpu-window", type=int, default=None,
                    help="memory window of the CPU runs (default: the workload's M, reduced only if the "
                         "FP64 history does not fit in host memory)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="leave out the config-3 batch measured beside c5")
    ap.add_argument("--config", default="c5", choices=["c5", "small", "c3", "c4", "ninv"],
                    help="c5: the benchmark workload; small: Ns=40, M=400 for profiler captures; "
                         "c3: 64 uneven runs in one launch; c4: adjoint gradients; ninv: 1/N expansion at NLO")
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--ns", type=int, default=None, help="override Ns of the c5/small workload (sweeps)")
    ap.add_argument("--m", type=int, default=None, help="override the memory window M (sweeps)")
    ap.add_argument("--memint-variant", type=int, default=None,
                    help="fix the mixed-precision memory-integral variant instead of autotuning")
    ap.add_argument("--sunset-grid", type=int, default=None, help="fix the sunset grid instead of autotuning")
    ap.add_argument("--batch-order", type=int, default=None, help="fix the run order of the batched grids (c3)")
    ap.add_argument("--memint-split", type=int, default=None, help="fix the split mode of the memory integrals")
    ap.add_argument("--memint-persistent", type=int, default=None,
                    help="1: persistent memory-integral grid (one CTA per SM taking items from a queue)")
    ap.add_argument("--sunset-variant", type=int, default=None,
                    help="fix the FP32 sunset variant (0: 1024, 1: 512 threads, 2: tensor cores)")
    ap.add_argument("--batch-overlap", type=int, default=None,
                    help="c3: fix the concurrent-group step (SMs of the second group's sunset; 0 = off)")
    args = ap.parse_args()
    if args.config == "c3" and args.impl == "ours":
        return run_batched(args)
    if args.config == "c4" and args.impl == "ours":
        return run_adjoint(args)
    if args.config == "ninv" and args.impl == "ours":
        return run_ninverse(args)
    if args.config == "small":
        CFG.update(SMALL)
    if args.ns:
        CFG["Ns"] = args.ns
    if args.m:
        CFG["M"] = args.m
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

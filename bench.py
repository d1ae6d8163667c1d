"""Benchmark: particle-steps/s of the GPU gravity / SPH engine on one GB300.

Default line (the headline): the direct-sum precision study at its largest
size.  Plummer sphere N = 2^20 (reference sampler, seed 1), eps = 0.04 /
N^(1/3), leapfrog KDK with dt = 1e-4, pair forces in mixed precision (f32
pairs on f64 tile centres, compensated sums), f64 kick/drift.  One step = one
KDK step (half-kick, drift, Hilbert sort + tile packing, all-pairs force,
half-kick).  The f64 state (134 MB) is larger than L2 and L2 is also flushed
between timed steps.

The same run also measures, under "extras" (one GPU, rank 0, N = 1 only),
every other workload of the engine with its own clocks, roofline, CPU
baseline and end-to-end figure:
  fp64       the FP64 form of the pair kernel at the same N (mixed vs FP64)
  plummer1k  the headless Plummer run: N = 1000, seed 42, eps 0.01, dt 1e-3,
             10^4 steps, exact f64 and mixed, drift against the oracle's run
  bh         Barnes-Hut KDK on two Plummer spheres, N = 2^22, theta 0.5:
             the parity walk (the reference's opening decisions) and the f32
             group walk (a refinement of each particle's node set)
  sph        grad-h SPH + BH gravity on the rho ~ 1/r gas sphere, N = 2^18,
             mixed and f64 pair arithmetic
  ensemble   512 Plummer systems of log-uniform N in [256, 16384], one launch
             per step, against one launch per system
  adjoint    N = 16384, 1000 steps, f64 checkpoints every 100: backward over
             forward, and the gradient against f64 central differences
Each of those also runs alone with --workload NAME (one JSON line of its own);
--workload precision runs the direct-sum precision study.

Arms:
  default          the engine (libgvs.so) on cuda:LOCAL_RANK
  --impl reference the reference's CPU algorithm (the C restatement in oracle/,
                   since the Rust reference cannot be built here) on all host
                   cores, timed on a bounded sample of the same workload.

Prints ONE JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: mixed vs FP64 at force rel err <=1e-6; adjoint/fwd"
UNIT = "particle-steps/s"
WORKLOADS = ("direct", "plummer1k", "bh", "sph", "ensemble", "adjoint", "precision", "device_ics")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gvs", choices=["gvs", "reference"])
    ap.add_argument("--n", type=int, default=None,
                    help="particles: 2^20 (direct), 2^22 (bh), 2^18 (sph) unless given")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--dt", type=float, default=1e-4)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "fp64", "fp64_exact"])
    ap.add_argument("--fp64-n", type=int, default=None,
                    help="N of the FP64 comparison (default: the headline N)")
    ap.add_argument("--cpu-targets", type=int, default=32768, help="targets in the bounded CPU sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the side measurements (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true", help="use the default kernel shape (profiling runs)")
    ap.add_argument("--workload", default="direct", choices=WORKLOADS,
                    help="direct (default headline); the others print their own line")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--sph-precision", default="both", choices=["both", "mixed", "f64"],
                    help="SPH workload: time both pair-arithmetic forms (and compare them), or one only")
    ap.add_argument("--nsys", type=int, default=512, help="systems in the ensemble workload")
    ap.add_argument("--adjoint-steps", type=int, default=1000, help="steps of the adjoint measurement")
    ap.add_argument("--adjoint-n", type=int, default=16384, help="particles of the adjoint measurement")
    ap.add_argument("--fd-dirs", type=int, default=2,
                    help="random directions of the adjoint's finite-difference check (f64 forward runs)")
    ap.add_argument("--seeds", default="1,2,3", help="precision study: Plummer seeds")
    ap.add_argument("--sizes", default="16,18,20", help="precision study: log2 N")
    a = ap.parse_args()
    if a.n is None:
        a.n = {"bh": 1 << 22, "sph": 1 << 18}.get(a.workload, 1 << 20)
    return a


# ---- distributed plumbing (replicas only: no data-path collective) -------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def replica_rate(units_per_rank: float, local_seconds: float, d: Dist) -> tuple[float, float]:
    """Whole-job rate of N independent replicas: every rank processed units_per_rank;
    the job takes as long as the slowest rank.  Returns (rate, max seconds)."""
    t = d.max(local_seconds)
    return units_per_rank * d.world / t, t


# ---- clocks sampler -------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([s.strip() for s in out.stdout.strip().split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---- peaks and traffic -------------------------------------------------------------
def hbm_peak_gbs():
    """HBM copy bandwidth measured on this machine (MEASURED_PEAKS.json beside this file), else
    the fallback figure of one earlier GB300 measurement; returns (GB/s, source)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback 6.8 TB/s"


class Peaks:
    """FP32 peak of this GPU: the FMA probe measured in this run (the denominator) and
    the nominal figure num_sms x 128 lanes x 2 flop x max SM clock beside it."""

    def __init__(self, ctx, device: int):
        self.ctx = ctx
        self.device = device
        self._fp32 = None
        self._nominal = None

    def fp32(self) -> float:
        if self._fp32 is None:
            self._fp32 = self.ctx.fp32_peak_tflops()
        return self._fp32

    def nominal(self) -> dict:
        if self._nominal is None:
            sms, mhz = None, None
            try:
                import torch
                sms = torch.cuda.get_device_properties(self.device).multi_processor_count
            except Exception:
                pass
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.max.sm",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
                mhz = float(out.stdout.strip())
            except Exception:
                pass
            tf = sms * 128 * 2 * mhz * 1e6 / 1e12 if sms and mhz else None
            self._nominal = {"num_sms": sms, "sm_max_mhz": mhz, "fp32_nominal_tflops": tf}
        return self._nominal

    def fp32_roofline(self, achieved_tflops: float, **extra) -> dict:
        peak = self.fp32()
        nom = self.nominal()
        r = {"bound": "fp32", "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
             "frac": achieved_tflops / peak if peak else None,
             "peak_source": "of measured FP32 FMA probe in this run (gvs_measure_fp32_peak)",
             "num_sms": nom["num_sms"], "fp32_nominal_tflops": nom["fp32_nominal_tflops"],
             "frac_of_nominal": achieved_tflops / nom["fp32_nominal_tflops"] if nom["fp32_nominal_tflops"] else None}
        r.update(extra)
        return r


def traffic(kernel: str, units: float):
    """DRAM bytes (read + write) of one launch of `kernel` that processes `units` (particles,
    or pairs for an all-pairs kernel), scaled from the ncu capture in profiles/traffic.json."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            t = json.load(fh)[kernel]
    except (OSError, KeyError, ValueError):
        return None, None
    scale = units / t["units"] if t.get("scaled", True) else 1.0
    return t["bytes"] * scale, t["source"]


def step_events(ctx, fn, steps: int, flush: bool = True) -> list:
    """Per-step CUDA-event times (ms) on the context stream, L2 flushed before each step."""
    ms = []
    for _ in range(steps):
        if flush:
            ctx.l2_flush()
        ctx.event(0)
        fn()
        ctx.event(1)
        ms.append(ctx.elapsed(0, 1))
    return ms


def pinned(n: int, names) -> dict:
    import torch
    return {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k in names}


def e2e_kdk_host(ctx, G, L, p, algo, prec, eps, theta, dt, steps):
    """End to end through the Integrator drop-in (gvs_kdk_step_host): x, v, a, m copied
    from pinned host arrays, one step, x, v, a copied back, every step."""
    names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass")
    host = pinned(p.count, names)
    for k in names:
        host[k][:] = getattr(p, k)
    lib = L.load()
    ptr = {k: host[k].ctypes.data for k in names}
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        L.check(lib.gvs_kdk_step_host(ctx.h, p.count, ptr["x"], ptr["y"], ptr["z"], ptr["vx"], ptr["vy"], ptr["vz"],
                                      ptr["ax"], ptr["ay"], ptr["az"], ptr["mass"], algo, prec, eps, theta, dt), ctx.h)
        ts.append(time.perf_counter() - t0)
    return {"value": p.count * steps / sum(ts), "unit": UNIT, "h2d_bytes_per_step": 10 * 8 * p.count,
            "d2h_bytes_per_step": 9 * 8 * p.count, "steps": steps,
            "how": "gvs_kdk_step_host (Integrator::step drop-in) on pinned host arrays, wall clock"}


# ---- the CPU reference arm ------------------------------------------------------------
def workload(n, seed):
    return {"workload": f"direct-sum KDK, Plummer N={n} (seed {seed}), eps=0.04/N^(1/3), dt=1e-4",
            "n": n, "seed": seed, "eps": 0.04 / n ** (1.0 / 3.0), "dt": 1e-4, "l2": "flushed between steps",
            "parallelism": "replicas (one independent system per GPU)"}


PREC = {"mixed": 3, "fp32": 2, "fp64": 1, "fp64_exact": 0}


def cpu_sample(n, seed, eps, targets, rng_seed=0):
    """Times the oracle's direct sum on `targets` targets against all n sources
    on all host cores; returns (particle-steps/s, cores, seconds, sample text)."""
    import oracle as O
    p = O.plummer(n, seed)
    idx = np.sort(np.random.default_rng(rng_seed).choice(n, size=min(targets, n), replace=False))
    cores = O.lib().orc_max_threads()
    O.bf_subset(p, eps, idx[: min(32, len(idx))])  # warm the threads
    t0 = time.perf_counter()
    O.bf_subset(p, eps, idx)
    dt = time.perf_counter() - t0
    step_s = dt * n / len(idx)  # one full force evaluation, extrapolated by target count
    return n / step_s, cores, dt, (f"{len(idx)} of {n} targets x {n} sources (one force evaluation, gather form, "
                                   f"all cores), extrapolated to all targets")


def cpu_serial_symmetric(n_full, seed, eps, n_sample=16384):
    """The reference's own loop form: BruteForce's serial j > i symmetric sum on one core,
    at a bounded N, extrapolated to n_full by the pair count."""
    import oracle as O
    p = O.plummer(n_sample, seed)
    t0 = time.perf_counter()
    O.bf_serial(p, eps)
    dt = time.perf_counter() - t0
    step_s = dt * (n_full / n_sample) ** 2
    return {"value": n_full / step_s, "unit": UNIT, "cores": 1, "kind": "port", "form": "serial symmetric j > i",
            "sample": f"one serial BruteForce evaluation at N={n_sample}, extrapolated by (N/{n_sample})^2",
            "seconds": dt}


def to_oracle(p):
    """The oracle's Particles with the same arrays (gas fields included)."""
    import oracle as O
    q = O.Particles(p.count)
    for a, b in (("x", "x"), ("y", "y"), ("z", "z"), ("vx", "vx"), ("vy", "vy"), ("vz", "vz"), ("mass", "mass"),
                 ("density", "density"), ("pressure", "pressure"), ("internal_energy", "u"),
                 ("smoothing_length", "h"), ("sound_speed", "cs"), ("alpha_visc", "alpha"),
                 ("particle_type", "ptype")):
        getattr(q, b)[:] = getattr(p, a)
    return q


def run_reference(a, d: Dist):
    if d.rank != 0:
        return
    w = workload(a.n, a.seed)
    vals = []
    for _ in range(max(1, a.warmup)):
        cpu_sample(a.n, a.seed, w["eps"], 256)
    last = None
    per_step_targets = max(256, a.cpu_targets // 16)
    for s in range(a.steps):
        v, cores, secs, sample = cpu_sample(a.n, a.seed, w["eps"], per_step_targets, rng_seed=s)
        vals.append(v)
        last = (cores, sample)
    v = float(np.median(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": a.n / v * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (reference Plummer sampler)", "impl": "reference",
            "config": w,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": last[0], "kind": "port", "sample": last[1],
                             "form": "gather (each target sums all sources), OpenMP over targets"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- the engine arm: the headline direct-sum line ------------------------------------------
def run_engine(a, d: Dist):
    import gravis_gb300 as G
    from gravis_gb300 import _lib as L
    w = workload(a.n, a.seed)
    prec = PREC[a.precision]
    ctx = G.Context(d.local)
    peaks = Peaks(ctx, d.local)
    p = G.PlummerSphere(a.n, seed=a.seed).generate()
    eps, dt = w["eps"], a.dt
    ctx.set_state(p)
    tune = ctx.autotune(prec, eps) if prec in (2, 3) and not a.no_autotune else None
    if tune is not None:
        tune["candidates"] = ctx.autotune_report()
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
    for _ in range(a.warmup):
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 1)
    ctx.sync()

    # -- device-resident timed region: K steps, per-step events, L2 flushed between
    ctx.profile(True)
    d.barrier()
    ctx.sync()
    wall0 = time.perf_counter()
    with Clocks(d.local) as clk:
        step_ms = step_events(ctx, lambda: ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 1), a.steps)
    ctx.sync()
    wall = time.perf_counter() - wall0
    prof = ctx.profile_read()
    ctx.profile(False)
    d.barrier()
    value, t_s = replica_rate(a.n * a.steps, sum(step_ms) * 1e-3, d)
    t_ms = t_s * 1e3

    # -- e2e through the Integrator drop-in with pinned host buffers
    q = G.Particles(a.n)
    ctx.get_state(q)
    q.mass[:] = p.mass
    d.barrier()
    e2e = e2e_kdk_host(ctx, G, L, q, G.ALGO_DIRECT, prec, eps, 0.0, dt, max(1, min(a.steps, 5)))
    e2e["value"], _ = replica_rate(a.n * e2e["steps"], a.n * e2e["steps"] / e2e["value"], d)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"mixed": "f32 pairs / f64 state", "fp32": "f32", "fp64": "f64",
                                           "fp64_exact": "f64"}[a.precision],
            "data": "synthetic (reference Plummer sampler, seed 1)", "config": w,
            "wall_s_timed_region": wall, "autotune": tune,
            "gpu_launches": int(prof["launches"]), "e2e": e2e, "clocks": clk.summary()}

    # -- roofline of the dominant kernel (the tiled f32 pair kernel)
    kernel_ms = prof["force_ms"] / max(1, prof["force_launches"])
    flops = prof["force_flops"] / max(1, prof["force_launches"])
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    tr, tr_src = traffic("k_direct32", float(a.n) * a.n)
    line["roofline"] = peaks.fp32_roofline(
        achieved, traffic=tr, traffic_source=tr_src, kernel="k_direct32 (mixed, f32x2 pairs)", kernel_ms=kernel_ms,
        flops_per_launch=flops, work_unit="20 flop per pair interaction, N^2 pairs per force evaluation",
        interactions_per_s=flops / 20.0 / (kernel_ms * 1e-3),
        near_field_tile_fraction=prof["near_tile_visits"] / max(1.0, prof["tile_visits"]))
    if d.rank == 0 and d.world == 1 and not a.no_extras:
        line["extras"] = headline_extras(ctx, G, L, a, p, eps, peaks)
        try:
            v, cores, secs, sample = cpu_sample(a.n, a.seed, eps, a.cpu_targets)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                    "seconds": secs, "form": "gather (each target sums all sources)",
                                    "serial_symmetric_1core": cpu_serial_symmetric(a.n, a.seed, eps)}
        except Exception as ex:  # the oracle must be built (build() does it)
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                                    "sample": f"unavailable: {ex}"}
    ctx.close()
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def headline_extras(ctx, G, L, a, p, eps, peaks) -> dict:
    extras = {}
    t0 = time.perf_counter()
    # every form of the pair kernel at the same N: rate (kernel time) and force error
    # against the exact f64 sum on a target subset
    n64 = a.fp64_n or a.n
    p64 = p if n64 == a.n else G.PlummerSphere(n64, seed=a.seed).generate()
    e64 = 0.04 / n64 ** (1.0 / 3.0)
    idx = np.sort(np.random.default_rng(123).choice(n64, size=min(n64, 1024), replace=False))
    ctx.set_state(p64)
    ref = ctx.direct_subset(idx, e64, G.PREC_FP64_EXACT)
    forms = {}
    for name, pr, reps in (("fp64", G.PREC_FP64, 1), ("fp32", G.PREC_FP32, 2), ("mixed", G.PREC_MIXED, 2)):
        ctx.set_state(p64)
        if reps > 1:
            ctx.compute_forces(G.ALGO_DIRECT, pr, e64)  # warm
        ctx.profile(True)
        for _ in range(reps):
            ctx.compute_forces(G.ALGO_DIRECT, pr, e64)
        pf = ctx.profile_read()
        ctx.profile(False)
        q = G.Particles(n64)
        ctx.get_state(q)
        got = q.acc()[idx]
        per = np.sqrt(((got - ref) ** 2).sum(1) / (ref ** 2).sum(1))
        forms[name] = {"interactions_per_s": pf["force_flops"] / 20.0 / (pf["force_ms"] * 1e-3),
                       "kernel_ms": pf["force_ms"] / max(1, pf["force_launches"]),
                       "acc_rel_rms_vs_exact_f64": float(np.sqrt(((got - ref) ** 2).sum() / (ref ** 2).sum())),
                       "acc_rel_max_vs_exact_f64": float(per.max())}
    extras["forms_same_n"] = dict(forms, n=n64, subset="1024 random targets, exact f64 sum on the GPU",
                                  mixed_vs_fp64=forms["mixed"]["interactions_per_s"] /
                                  forms["fp64"]["interactions_per_s"])
    extras["headline_extras_s"] = time.perf_counter() - t0
    for name, fn in (("plummer1k", wl_plummer1k), ("bh", wl_bh), ("sph", wl_sph), ("ensemble", wl_ensemble),
                     ("adjoint", wl_adjoint), ("device_ics", wl_device_ics)):
        t0 = time.perf_counter()
        try:
            extras[name] = fn(ctx, G, L, a, peaks, extra=True)
        except Exception as ex:  # one workload failing must not lose the headline line
            extras[name] = {"error": f"{type(ex).__name__}: {ex}"}
        extras[name]["bench_seconds"] = time.perf_counter() - t0
    return extras


# ---- workloads ---------------------------------------------------------------------------
def wl_device_ics(ctx, G, L, a, peaks, extra=False) -> dict:
    """PlummerSphere::generate on the GPU (gvs_ic_plummer_device) against the host generator
    (gvs_ic_plummer, one core) at the headline's N and seed: wall time of each call, and the
    largest difference relative to the largest coordinate."""
    n, seed = a.n, a.seed
    ctx.ic_plummer_device(min(n, 4096), seed)  # warm: module load, first allocations
    t0 = time.perf_counter()
    ctx.ic_plummer_device(n, seed)
    t1 = time.perf_counter()
    q = G.Particles(n)
    ctx.get_state(q)
    t2 = time.perf_counter()
    host = G.PlummerSphere(n, seed=seed).generate()
    t3 = time.perf_counter()
    worst = max(float(np.abs(getattr(q, f) - getattr(host, f)).max()) / float(np.abs(getattr(host, f)).max())
                for f in ("x", "y", "z", "vx", "vy", "vz"))
    return {"n": n, "seed": seed, "device_ms": 1e3 * (t1 - t0), "host_ms": 1e3 * (t3 - t2),
            "speedup": (t3 - t2) / max(t1 - t0, 1e-9), "max_rel_diff_vs_host": worst,
            "how": "wall clock around each call; the device call ends with the state resident (no copy)"}



def wl_plummer1k(ctx, G, L, a, peaks, extra=False) -> dict:
    """The headless plummer run: N=1000, seed 42, eps=0.01, dt=1e-3, 10^4 KDK steps."""
    n, eps, dt = 1000, 0.01, 1e-3
    steps = 10000 if extra else max(100, a.steps)
    p = G.PlummerSphere(n, seed=42).generate()
    fixture = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "config1_oracle.json")) as fh:
            fixture = json.load(fh)
    except OSError:
        pass
    out = {}
    for name, prec in (("fp64_exact", G.PREC_FP64_EXACT), ("mixed", G.PREC_MIXED)):
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        e0 = ctx.diagnostics(eps).total_energy
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 2)  # captures the step graph
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        ctx.sync()
        with Clocks(0) as clk:
            ctx.event(0)
            ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, steps)
            ctx.event(1)
            t = ctx.elapsed(0, 1)
        dg = ctx.diagnostics(eps)
        r = {"value": n * steps / (t * 1e-3), "ms_per_step": t / steps, "clocks": clk.summary(),
             "rel_energy_drift": abs((dg.total_energy - e0) / e0), "momentum": dg.momentum_magnitude()}
        if fixture and steps == 10000:
            rows = fixture["rows"]
            r["oracle_rel_energy_drift"] = abs((rows[-1]["total_energy"] - rows[0]["total_energy"]) /
                                               rows[0]["total_energy"])
            if name == "fp64_exact":
                import hashlib
                q = G.Particles(n)
                ctx.get_state(q)
                h = hashlib.sha256()
                for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
                    h.update(np.ascontiguousarray(getattr(q, f), dtype="<f8").tobytes())
                r["final_state_bit_identical_to_oracle"] = h.hexdigest() == rows[-1]["state_sha256"]
        out[name] = r
    # roofline: pair work of the mixed step against the FP32 peak (this size is launch- and
    # latency-bound: 10^6 pairs per step)
    ach = 20.0 * n * n / (out["mixed"]["ms_per_step"] * 1e-3) / 1e12
    roof = peaks.fp32_roofline(ach, traffic=None, kernel="the whole mixed KDK step (graph replay)",
                               note="N=1000 is latency- and launch-bound: a step is a chain of small kernels")
    tr, tr_src = traffic("plummer1k_step_exact", float(n) * n)
    out["fp64_exact"]["traffic_per_step"] = {"bytes": tr, "source": tr_src,
                                             "note": "cold-cache (ncu): the 24 MB of f64 terms of one step"}
    # end to end: the Integrator drop-in with host arrays, every step
    q = p.copy()
    ctx.set_state(q)
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
    ctx.get_state(q)
    e2e = e2e_kdk_host(ctx, G, L, q, G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, min(1000, steps))
    # the reference's CPU path: serial symmetric BruteForce + KDK on one core, a bounded run
    import oracle as O
    oq = O.plummer(n, 42)
    O.bf_serial(oq, eps)
    ks = 400
    t0 = time.perf_counter()
    O.kdk_steps(oq, O.gravity(O.GRAV_BF, eps), dt, ks)
    tc = time.perf_counter() - t0
    res = {"value": out["mixed"]["value"], "unit": UNIT, "ms_per_step": out["mixed"]["ms_per_step"],
           "dtype": "f32 pairs / f64 state", "steps": steps,
           "config": {"workload": f"headless plummer: N={n} seed 42, eps={eps}, dt={dt}, {steps} KDK steps, "
                                  "each step a CUDA-graph replay", "n": n,
                      "l2": "resident (a 1000-particle state is 100 KB; a real run keeps it in L2)"},
           "fp64_exact": out["fp64_exact"], "mixed": out["mixed"], "clocks": out["mixed"]["clocks"],
           "roofline": roof, "e2e": e2e,
           "cpu_baseline": {"value": n * ks / tc, "unit": UNIT, "cores": 1, "kind": "port",
                            "sample": f"{ks} KDK steps of the same system, serial symmetric BruteForce"}}
    return res


def wl_bh(ctx, G, L, a, peaks, extra=False) -> dict:
    """Barnes-Hut KDK, two Plummer spheres (seed 7), theta, eps 1e-3, dt 5e-4."""
    n = a.n if not extra else 1 << 22
    steps = a.steps if not extra else 3
    warm = a.warmup if not extra else 1
    theta, eps, dt = a.theta, 1e-3, 5e-4
    p = G.collision(n, seed=7)
    forms = {}
    for name, prec, parity in (("parity", G.PREC_MIXED, "the reference's opening decisions (within 1e-6 of the "
                                                         "oracle's BarnesHut)"),
                               ("group", G.PREC_FP32, "unpinned: a refinement of each particle's node set")):
        ctx.set_bh_walk(-1)
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_BH, prec, eps, theta)
        for _ in range(warm):
            ctx.kdk_steps(G.ALGO_BH, prec, eps, theta, dt, 1)
        ctx.profile(True)
        with Clocks(0) as clk:
            ms = step_events(ctx, lambda: ctx.kdk_steps(G.ALGO_BH, prec, eps, theta, dt, 1), steps)
        prof = ctx.profile_read()
        ctx.profile(False)
        walk_ms = prof["force_ms"] / max(1, prof["force_launches"])
        terms = (prof["bh_walk_terms"] + prof["bh_group_interactions"]) / max(1, prof["force_launches"])
        kern = "k_walk<2> (mixed per-particle walk)" if name == "parity" else "k_walk_group (f32 group walk)"
        tr, tr_src = traffic("k_walk_mixed" if name == "parity" else "k_walk_group", float(n))
        roof = peaks.fp32_roofline(terms * 20.0 / (walk_ms * 1e-3) / 1e12, traffic=tr, traffic_source=tr_src,
                                   kernel=kern, kernel_ms=walk_ms, terms_per_particle=terms / n,
                                   work_unit="20 flop per node or particle term summed")
        hbm, hsrc = hbm_peak_gbs()
        step_ms = sum(ms) / steps
        roof["hbm_algorithmic"] = {"bytes_per_particle_step": 252 + 96, "achieved_gbs": n * 348 / (step_ms * 1e-3) / 1e9,
                                   "peak": hbm, "peak_source": hsrc}
        forms[name] = {"value": n * steps / (sum(ms) * 1e-3), "ms_per_step": step_ms, "walk_ms": walk_ms,
                       "parity": parity, "clocks": clk.summary(), "roofline": roof,
                       "gpu_launches_per_step": prof["launches"] / steps}
    # accuracy of both walks on the final state: per-particle error against the exact f64 sum
    idx = np.sort(np.random.default_rng(1).choice(n, 1024, replace=False))
    ref = ctx.direct_subset(idx, eps)
    for name, prec in (("parity", G.PREC_MIXED), ("group", G.PREC_FP32)):
        ctx.compute_forces(G.ALGO_BH, prec, eps, theta)
        q = G.Particles(n)
        ctx.get_state(q)
        got = q.acc()[idx]
        forms[name]["per_particle_rms_rel_err_vs_exact_f64_direct"] = float(
            np.sqrt((((got - ref) ** 2).sum(1) / (ref ** 2).sum(1)).mean()))
    # end to end through the Integrator drop-in, parity walk
    q = G.Particles(n)
    ctx.get_state(q)
    q.mass[:] = p.mass
    e2e = e2e_kdk_host(ctx, G, L, q, G.ALGO_BH, G.PREC_MIXED, eps, theta, dt, 2)
    res = {"value": forms["parity"]["value"], "unit": UNIT, "ms_per_step": forms["parity"]["ms_per_step"],
           "dtype": "f32 terms on float-float separations / f64 state", "steps": steps,
           "config": {"workload": f"Barnes-Hut KDK, two Plummer spheres N={n} seed 7, theta={theta}, eps={eps}, "
                                  f"dt={dt}", "n": n, "theta": theta, "l2": "flushed between steps"},
           "walks": forms, "clocks": forms["parity"]["clocks"], "roofline": forms["parity"]["roofline"],
           "e2e": e2e, "headline": "the parity walk; the group walk is faster but parity-unpinned"}
    if not a.no_extras or extra:
        res["cpu_baseline"] = cpu_bh_sample(G, theta, eps)
    if extra:
        res["parity_other_configs"] = bh_parity_configs(ctx, G, eps, dt)
    return res


def bh_parity_configs(ctx, G, eps, dt, steps=2) -> dict:
    """The parity walk's KDK step at the workload's other sizes and opening angles
    (N = 2^22, 2^24; theta = 0.5, 0.7), on collision ICs generated on the device."""
    out = {}
    for n, theta in ((1 << 22, 0.7), (1 << 24, 0.5), (1 << 24, 0.7)):
        ctx.ic_collision_device(n, 7)
        ctx.compute_forces(G.ALGO_BH, G.PREC_MIXED, eps, theta)
        ctx.kdk_steps(G.ALGO_BH, G.PREC_MIXED, eps, theta, dt, 1)  # warm
        ctx.profile(True)
        ms = step_events(ctx, lambda: ctx.kdk_steps(G.ALGO_BH, G.PREC_MIXED, eps, theta, dt, 1), steps)
        prof = ctx.profile_read()
        ctx.profile(False)
        launches = max(1, prof["force_launches"])
        out[f"n{n}_theta{theta}"] = {"value": n * steps / (sum(ms) * 1e-3), "unit": UNIT,
                                     "ms_per_step": sum(ms) / steps, "walk_ms": prof["force_ms"] / launches,
                                     "terms_per_particle": prof["bh_walk_terms"] / launches / n}
    out["how"] = f"{steps} CUDA-event-timed KDK steps after one warm step, L2 flushed before each"
    return out


def cpu_bh_sample(G, theta, eps, n=1 << 20):
    """The oracle's BarnesHut (serial build, threaded walk) for one force evaluation
    of the same two-sphere system at a bounded N."""
    import oracle as O
    q = to_oracle(G.collision(n, seed=7))
    t0 = time.perf_counter()
    O.bh(q, eps, theta)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": O.lib().orc_max_threads(), "kind": "port",
            "sample": f"one BarnesHut force evaluation (serial tree build + threaded walk) of the same collision "
                      f"ICs at N={n}, theta={theta}; the step's KDK update is not included"}


def wl_sph(ctx, G, L, a, peaks, extra=False) -> dict:
    n = a.n if not extra else 1 << 18
    steps = a.steps if not extra else 3
    warm = a.warmup if not extra else 2
    p = G.gas_sphere_1r(n)
    eps = 0.3 * (4.0 / 3.0 * np.pi / n) ** (1.0 / 3.0)
    theta = a.theta
    sph = G.SphSolver(ctx)
    gas_fields = ("density", "pressure", "internal_energy", "du_dt", "smoothing_length", "sound_speed", "alpha_visc")

    def upload(q):
        ctx.set_state(q)
        ctx.set_accelerations(q)
        ctx._ck(ctx._lib.gvs_set_gas(ctx.h, *(G.engine._ptr(getattr(q, f)) for f in gas_fields)))

    def sph_only(prec):
        """one SphSolver::compute on the initial state, SPH terms only"""
        upload(p)
        sph.params.precision = prec
        ctx._ck(ctx._lib.gvs_sph_compute(ctx.h, C.byref(sph.params), None, None, None, None))
        q = G.Particles(n)
        ctx.get_state(q)
        ctx.get_gas(q)
        return q

    def start(prec):
        upload(p)
        sph.params.precision = prec
        ctx.compute_forces(G.ALGO_BH, G.PREC_FP32, eps, theta)
        ctx._ck(ctx._lib.gvs_sph_compute(ctx.h, C.byref(sph.params), None, None, None, None))
        dtc = C.c_double()
        ctx._ck(ctx._lib.gvs_sph_timestep(ctx.h, C.byref(sph.params), C.byref(dtc)))
        return dtc.value

    def step(dt):
        dtc = C.c_double()
        ctx._ck(ctx._lib.gvs_sph_step(ctx.h, C.byref(sph.params), G.ALGO_BH, G.PREC_FP32, eps, theta, dt,
                                      C.byref(dtc)))
        return min(dtc.value, 1.5 * dt)

    def timed(prec):
        dt = [start(prec)]
        for _ in range(warm):
            dt[0] = step(dt[0])
        ctx.profile(True)

        def one():
            dt[0] = step(dt[0])
        with Clocks(0) as clk:
            ms = step_events(ctx, one, steps)
        prof = ctx.profile_read()
        ctx.profile(False)
        return sum(ms), clk.summary(), prof

    forms = [a.sph_precision] if a.sph_precision != "both" and not extra else ["f64", "mixed"]
    res = {"unit": UNIT, "steps": steps}
    times = {}
    for f in forms:
        prec = G.PREC_MIXED if f == "mixed" else G.PREC_FP64_EXACT
        t, clk, prof = timed(prec)
        times[f] = (t, clk, prof)
    main = "mixed" if "mixed" in times else forms[0]
    t, clk, prof = times[main]
    res.update({"value": n * steps / (t * 1e-3), "ms_per_step": t / steps,
                "dtype": "f32 SPH pair terms (mixed) / f64 state / f32 BH walk" if main == "mixed" else "f64 SPH",
                "config": {"workload": f"grad-h SPH + BH gravity, rho~1/r gas sphere N={n}, u=0.05, Wendland C2, "
                                       f"eta=1.2, theta={theta}, eps={eps:.3g}, CFL 0.3", "n": n,
                           "l2": "flushed between steps"},
                "clocks": clk, "gpu_launches_per_step": prof["launches"] / steps})
    if "f64" in times and main == "mixed":
        t64 = times["f64"][0]
        res["f64_exact"] = {"value": n * steps / (t64 * 1e-3), "ms_per_step": t64 / steps,
                            "what": "the same steps with the reference's f64 SPH arithmetic"}
        res["mixed_over_f64"] = t64 / t
        qe = sph_only(G.PREC_FP64_EXACT)
        qm = sph_only(G.PREC_MIXED)

        def rel(f):
            x, y = getattr(qm, f), getattr(qe, f)
            return float(np.sqrt(((x - y) ** 2).sum() / max((y ** 2).sum(), 1e-300)))
        res["mixed_vs_f64_rel_rms"] = {f: rel(f) for f in ("density", "smoothing_length", "ax", "ay", "az", "du_dt")}
    # roofline per the algorithmic bytes of one SPH step (density 120 B, forces 160 B,
    # neighbour rows 840 B, KDK 120 B per particle)
    hbm, hbm_src = hbm_peak_gbs()
    gbs = n * 1240.0 / (t / steps * 1e-3) / 1e9
    tr, tr_src = traffic("sph_step_mixed", float(n))
    res["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                       "traffic": tr, "traffic_source": tr_src, "traffic_scope": "every kernel of one step",
                       "bytes_per_particle_step": 1240, "peak_source": hbm_src,
                       "kernel": "the whole SPH step (neighbour search, density, forces, BH gravity, KDK)",
                       "note": "the SPH kernels are issue- and latency-bound well below this roofline "
                               "(neighbour walk, f32 pair gathers); their ncu figures are in profiles/"}
    # end to end: host arrays in and out every step (set_state + set_gas, step_with_sph,
    # get_state + get_gas)
    q = G.Particles(n)
    ctx.get_state(q)
    ctx.get_gas(q)
    q.mass[:] = p.mass
    q.particle_type[:] = p.particle_type
    names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass") + gas_fields
    host = pinned(n, names)
    for k in names:
        host[k][:] = getattr(q, k)
    pt = np.ascontiguousarray(p.particle_type)
    hp = {k: host[k].ctypes.data for k in names}
    lib = ctx._lib
    dtc = C.c_double()
    dt = start(G.PREC_MIXED)
    ts = []
    for _ in range(2):
        t0 = time.perf_counter()
        L.check(lib.gvs_set_state(ctx.h, n, hp["x"], hp["y"], hp["z"], hp["vx"], hp["vy"], hp["vz"], hp["mass"],
                                  pt.ctypes.data, hp["internal_energy"], hp["smoothing_length"], hp["alpha_visc"]),
                ctx.h)
        L.check(lib.gvs_set_accelerations(ctx.h, hp["ax"], hp["ay"], hp["az"]), ctx.h)
        L.check(lib.gvs_set_gas(ctx.h, *(hp[f] for f in gas_fields)), ctx.h)
        L.check(lib.gvs_sph_step(ctx.h, C.byref(sph.params), G.ALGO_BH, G.PREC_FP32, eps, theta, dt, C.byref(dtc)),
                ctx.h)
        L.check(lib.gvs_get_state(ctx.h, hp["x"], hp["y"], hp["z"], hp["vx"], hp["vy"], hp["vz"], hp["ax"], hp["ay"],
                                  hp["az"]), ctx.h)
        L.check(lib.gvs_get_gas(ctx.h, *(hp[f] for f in gas_fields)), ctx.h)
        ts.append(time.perf_counter() - t0)
        dt = min(dtc.value, 1.5 * dt)
    res["e2e"] = {"value": n * len(ts) / sum(ts), "unit": UNIT, "h2d_bytes_per_step": (10 + 7 + 3) * 8 * n + n,
                  "d2h_bytes_per_step": (9 + 7) * 8 * n, "steps": len(ts),
                  "how": "gvs_set_state/set_accelerations/set_gas, gvs_sph_step, gvs_get_state/get_gas on pinned "
                         "host arrays, wall clock"}
    if not a.no_extras or extra:
        res["cpu_baseline"] = cpu_sph_sample(G, n=n)
    if extra:  # the workload's larger size, mixed, a bounded run
        import copy
        b = copy.copy(a)
        b.n, b.steps, b.warmup, b.sph_precision, b.no_extras = 1 << 20, 3, 2, "mixed", True
        r20 = wl_sph(ctx, G, L, b, peaks, extra=False)
        res[f"n{b.n}"] = {k: r20[k] for k in ("value", "ms_per_step", "clocks", "roofline", "e2e", "config")
                          if k in r20}
    return res


def cpu_sph_sample(G, n=1 << 18):
    """The oracle's SphSolver::compute (neighbours, density, forces) once on the same
    gas sphere."""
    import oracle as O
    q = to_oracle(G.gas_sphere_1r(n))
    s = O.Sph()
    t0 = time.perf_counter()
    s.compute(q)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": O.lib().orc_max_threads(), "kind": "port",
            "sample": f"one SphSolver::compute of the rho~1/r sphere at N={n} (threaded neighbour search, serial "
                      f"density and forces as in the reference; no gravity, no KDK update)"}


def wl_ensemble(ctx, G, L, a, peaks, extra=False) -> dict:
    from gravis_gb300.engine import plummer_ensemble
    import torch
    nsys = a.nsys
    steps = a.steps if not extra else 10
    sizes = G.ensemble_sizes(nsys, seed=2024)
    p = plummer_ensemble(sizes)
    n, eps, dt = p.count, 0.01, 1e-3
    sum_n2 = float((sizes.astype(np.float64) ** 2).sum())
    ctx.set_state(p)
    ctx.ensemble_setup(sizes, eps)
    ctx.ensemble_forces()
    ctx.ensemble_kdk_steps(dt, max(2, a.warmup), True)
    ctx.sync()
    with Clocks(0) as clk:
        ctx.event(0)
        ctx.ensemble_kdk_steps(dt, steps, True)
        ctx.event(1)
        t = ctx.elapsed(0, 1)
    # kernel time of the pair kernel (profiled force evaluations)
    ctx.profile(True)
    for _ in range(3):
        ctx.ensemble_forces()
    pf = ctx.profile_read()
    ctx.profile(False)
    kern_ms = pf["force_ms"] / max(1, pf["force_launches"])
    # the same systems, one single-system context each; timed with CUDA events: a start
    # event on the first context's stream that every other stream waits for, and an end
    # event that waits for every stream's last step
    ctxs, o = [], 0
    for m in sizes:
        q = G.Particles(int(m))
        for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
            getattr(q, f)[:] = getattr(p, f)[o:o + m]
        o += m
        c = G.Context(0)
        c.set_state(q)
        c.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
        ctxs.append(c)
    streams = [torch.cuda.ExternalStream(c.stream()) for c in ctxs]

    def timed_all(launch, k):
        for c in ctxs:
            c.sync()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(streams[0])
        for s in streams[1:]:
            s.wait_event(e0)
        launch(k)
        for s in streams[1:]:
            ev = torch.cuda.Event()
            ev.record(s)
            streams[0].wait_event(ev)
        e1.record(streams[0])
        e1.synchronize()
        return e0.elapsed_time(e1)

    for c in ctxs:  # warm: captures each system's step graph
        c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 2)

    def per_step_calls(k):
        for _ in range(k):
            for c in ctxs:
                c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 1)

    def graphs(k):
        for c in ctxs:
            c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, k)

    kb, kg = 2, max(2, min(steps, 10))
    tb = timed_all(per_step_calls, kb)
    tg = timed_all(graphs, kg)
    for c in ctxs:
        c.close()
    v, vb, vg = n * steps / (t * 1e-3), n * kb / (tb * 1e-3), n * kg / (tg * 1e-3)
    ach = 20.0 * sum_n2 / (kern_ms * 1e-3) / 1e12
    tr, tr_src = traffic("k_direct32_items", sum_n2)
    res = {"value": v, "unit": UNIT, "ms_per_step": t / steps, "dtype": "f32 pairs / f64 state", "steps": steps,
           "config": {"workload": f"{nsys} Plummer systems, N_i log-uniform [256, 16384] (seed 2024), seeds 1000+i, "
                                  f"eps={eps}, dt={dt}, CUDA-graph steps", "n_total": n, "sum_n2": sum_n2,
                      "l2": "not flushed (steps replayed back to back; the 99 MB state is near L2 size)"},
           "clocks": clk.summary(),
           "roofline": peaks.fp32_roofline(ach, traffic=tr, traffic_source=tr_src,
                                           kernel="k_direct32_items (batched pair kernel)", kernel_ms=kern_ms,
                                           work_unit="20 flop per pair, sum N_i^2 pairs per evaluation"),
           "separate_systems": {"value": vb, "ms_per_step": tb / kb,
                                "how": "one single-system context per system, each step all systems in turn "
                                       "(CUDA events across the contexts' streams)"},
           "separate_systems_graphs": {"value": vg, "ms_per_step": tg / kg,
                                       "how": "one context per system, each runs its steps as CUDA-graph replays on "
                                              "its own stream, systems launched in turn (CUDA events)"},
           "batched_over_separate_per_step_calls": v / vb, "batched_over_separate_graphs": v / vg,
           "batched_over_separate": v / max(vb, vg)}
    # end to end: the whole ensemble's state in and out of pinned host arrays every step
    names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass")
    q = G.Particles(n)
    ctx.get_state(q)
    q.mass[:] = p.mass
    host = pinned(n, names)
    for k in names:
        host[k][:] = getattr(q, k)
    hp = {k: host[k].ctypes.data for k in names}
    lib = ctx._lib
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        L.check(lib.gvs_set_state(ctx.h, n, hp["x"], hp["y"], hp["z"], hp["vx"], hp["vy"], hp["vz"], hp["mass"],
                                  None, None, None, None), ctx.h)
        L.check(lib.gvs_set_accelerations(ctx.h, hp["ax"], hp["ay"], hp["az"]), ctx.h)
        ctx.ensemble_kdk_steps(dt, 1, False)
        L.check(lib.gvs_get_state(ctx.h, hp["x"], hp["y"], hp["z"], hp["vx"], hp["vy"], hp["vz"], hp["ax"], hp["ay"],
                                  hp["az"]), ctx.h)
        ts.append(time.perf_counter() - t0)
    res["e2e"] = {"value": n * len(ts) / sum(ts), "unit": UNIT, "h2d_bytes_per_step": 10 * 8 * n,
                  "d2h_bytes_per_step": 9 * 8 * n, "steps": len(ts),
                  "how": "gvs_set_state/set_accelerations, gvs_ensemble_kdk_steps(1), gvs_get_state on pinned host "
                         "arrays, wall clock"}
    # the reference's CPU path: the oracle's direct sum system by system on all cores, a bounded sample
    import oracle as O
    o, done, t_cpu = 0, 0, 0.0
    offs = np.concatenate([[0], np.cumsum(sizes)])
    for i in range(nsys):
        m = int(sizes[i])
        if t_cpu > 3.0:
            break
        q = O.Particles(m)
        for f in ("x", "y", "z", "mass"):
            getattr(q, f)[:] = getattr(p, f)[offs[i]:offs[i] + m]
        t0 = time.perf_counter()
        O.bf_gather(q, eps)
        t_cpu += time.perf_counter() - t0
        done += m
    res["cpu_baseline"] = {"value": done / t_cpu, "unit": UNIT, "cores": O.lib().orc_max_threads(), "kind": "port",
                           "sample": f"one force evaluation of the first systems ({done} particles), gather form on "
                                     "all cores; the KDK update is not included"}
    return res


def wl_adjoint(ctx, G, L, a, peaks, extra=False) -> dict:
    r = adjoint_ratio(ctx, G, n=a.adjoint_n, steps=a.adjoint_steps, every=100, fd_dirs=a.fd_dirs,
                      check_fp64=not extra)
    res = {"value": r["adjoint_over_forward"], "unit": "backward/forward", "higher_is_better": False,
           "adjoint": r, "clocks": r.pop("clocks")}
    # the fused force + VJP kernel against the FP32 peak (about 35 FP32 lane ops per pair;
    # counted here at the 20-flop convention of the force)
    n = a.adjoint_n
    ach = 20.0 * n * n / (r["vjp_kernel_ms"] * 1e-3) / 1e12
    tr, tr_src = traffic("k_force_vjp32", float(n) * n)
    res["roofline"] = peaks.fp32_roofline(ach, traffic=tr, traffic_source=tr_src,
                                          kernel="k_force_vjp32 (fused force + VJP)", kernel_ms=r["vjp_kernel_ms"],
                                          work_unit="20 flop per pair (the force's convention)")
    return res


def adjoint_ratio(ctx, G, n=16384, steps=1000, every=100, seed=42, eps=0.01, dt=1e-3, check_fp64=True, fd_dirs=2):
    """Adjoint workload: L = sum m |x(T) - x*|^2 for a Plummer sphere; cost of the
    backward sweep over the cost of the plain forward run, the mixed-precision gradient
    against the f64 adjoint, and against f64 central differences along random directions
    of (x0, v0, m)."""
    p = G.PlummerSphere(n, seed=seed).generate()

    def final_x(q0, prec):
        ctx.set_state(q0)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, steps)
        q = G.Particles(n)
        ctx.get_state(q)
        return np.stack([q.x, q.y, q.z], 1)

    xstar = final_x(p, G.PREC_MIXED) + 0.01 * np.random.default_rng(seed + 1).standard_normal((n, 3))

    def loss(q0):
        x = final_x(q0, G.PREC_FP64)
        return float((q0.mass[:, None] * (x - xstar) ** 2).sum())

    def run(prec):
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 2)  # captures the step graph
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        ctx.sync()
        ctx.event(2)
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, steps)
        ctx.event(3)
        fwd_plain = ctx.elapsed(2, 3)
        ctx.set_state(p)
        ctx.event(4)
        ctx.adjoint_forward(prec, eps, dt, steps, every)
        ctx.event(5)
        fwd_ck = ctx.elapsed(4, 5)
        q = G.Particles(n)
        ctx.get_state(q)
        x = np.stack([q.x, q.y, q.z], 1)
        ctx.profile(True)
        ctx.event(6)
        g = ctx.adjoint_backward(2.0 * p.mass[:, None] * (x - xstar))
        ctx.event(7)
        bwd = ctx.elapsed(6, 7)
        pf = ctx.profile_read()
        ctx.profile(False)
        g["m"] = g["m"] + ((x - xstar) ** 2).sum(1)  # the loss's own mass dependence
        return fwd_plain, fwd_ck, bwd, g, pf["vjp_ms"] / max(1, pf["vjp_launches"])

    with Clocks(0) as clk:
        f_plain, f_ck, bwd, g, vjp_ms = run(G.PREC_MIXED)
    out = {"workload": f"Plummer N={n} seed {seed}, eps={eps}, dt={dt}, {steps} steps, f64 checkpoints every {every}",
           "forward_ms": f_plain, "forward_with_checkpoints_ms": f_ck, "backward_ms": bwd,
           "adjoint_over_forward": bwd / f_plain, "vjp_kernel_ms": vjp_ms, "clocks": clk.summary()}
    g64 = None
    if check_fp64:
        _, _, bwd64, g64, _ = run(G.PREC_FP64)
        out["grad_rel_err_mixed_vs_fp64_adjoint"] = {
            k: float(np.linalg.norm(g[k] - g64[k]) / np.linalg.norm(g64[k])) for k in ("x", "v", "m")}
        out["fp64_backward_ms"] = bwd64
    if fd_dirs > 0:
        rng = np.random.default_rng(7)
        delta = 1e-6
        errs, errs64 = [], []
        for _ in range(fd_dirs):
            ux, uv, um = rng.standard_normal((n, 3)), rng.standard_normal((n, 3)), rng.standard_normal(n) * p.mass
            qs = []
            for s in (1.0, -1.0):
                q = p.copy()
                q.x += s * delta * ux[:, 0]; q.y += s * delta * ux[:, 1]; q.z += s * delta * ux[:, 2]
                q.vx += s * delta * uv[:, 0]; q.vy += s * delta * uv[:, 1]; q.vz += s * delta * uv[:, 2]
                q.mass += s * delta * um
                qs.append(loss(q))
            fd = (qs[0] - qs[1]) / (2 * delta)
            ad = float((g["x"] * ux).sum() + (g["v"] * uv).sum() + (g["m"] * um).sum())
            errs.append(abs(ad - fd) / abs(fd))
            if g64 is not None:
                ad64 = float((g64["x"] * ux).sum() + (g64["v"] * uv).sum() + (g64["m"] * um).sum())
                errs64.append(abs(ad64 - fd) / abs(fd))
        out["fd_check"] = {"directions": fd_dirs, "step": delta, "max_rel_err": float(max(errs)),
                           "median_rel_err": float(np.median(errs)), "bar": 1e-5,
                           "what": "mixed-precision adjoint directional derivative along random (x0, v0, m) "
                                   "directions against f64 central differences of the f64 forward run"}
        if errs64:
            out["fd_check_fp64_adjoint"] = {"max_rel_err": float(max(errs64)),
                                            "median_rel_err": float(np.median(errs64)),
                                            "what": "the f64 adjoint along the same directions"}
    return out


def wl_precision(ctx, G, L, a, peaks, extra=False) -> dict:
    """The direct-sum precision study: N in sizes x seeds x {FP64, FP32, mixed}; one force
    evaluation (error against the exact f64 sum on a target subset) plus 100 KDK steps at
    dt = 1e-4 (energy error from the f64 diagnostics).  FP64 100-step runs are made where
    they take under a minute (the FP64 pipe of this GPU runs the N = 2^20 form at ~33 s per
    evaluation); the FP64 force error is measured at every size."""
    sizes = [1 << int(s) for s in a.sizes.split(",")]
    seeds = [int(s) for s in a.seeds.split(",")]
    rows = []
    for n in sizes:
        eps = 0.04 / n ** (1.0 / 3.0)
        for seed in seeds:
            p = G.PlummerSphere(n, seed=seed).generate()
            ctx.set_state(p)
            idx = np.sort(np.random.default_rng(seed).choice(n, size=min(n, 4096), replace=False))
            ref = ctx.direct_subset(idx, eps, G.PREC_FP64_EXACT)
            for name, prec in (("fp64", G.PREC_FP64), ("fp32", G.PREC_FP32), ("mixed", G.PREC_MIXED)):
                ctx.set_state(p)
                ctx.profile(True)
                ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
                pf = ctx.profile_read()
                ctx.profile(False)
                q = G.Particles(n)
                ctx.get_state(q)
                got = q.acc()[idx]
                per = np.sqrt(((got - ref) ** 2).sum(1) / (ref ** 2).sum(1))
                row = {"n": n, "seed": seed, "form": name,
                       "acc_rel_rms": float(np.sqrt(((got - ref) ** 2).sum() / (ref ** 2).sum())),
                       "acc_rel_max": float(per.max()), "force_ms": pf["force_ms"]}
                step_cost_s = pf["force_ms"] * 1e-3 * 100
                if name != "fp64" or step_cost_s < 60.0:
                    e0 = ctx.diagnostics(eps).total_energy
                    ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, 1e-4, 100)
                    e1 = ctx.diagnostics(eps).total_energy
                    row["energy_rel_err_100_steps"] = float(abs((e1 - e0) / e0))
                rows.append(row)
    return {"value": None, "unit": "relative error", "rows": rows,
            "config": {"workload": "direct-sum precision study: Plummer (reference sampler), eps = 0.04/N^(1/3), "
                                   "one force evaluation + 100 KDK steps at dt = 1e-4", "sizes": sizes,
                       "seeds": seeds, "subset": "4096 random targets, exact f64 sum on the GPU"}}


def run_workload(a, d):
    """Secondary workloads (one JSON line each; the default run is the direct sum)."""
    import gravis_gb300 as G
    from gravis_gb300 import _lib as L
    ctx = G.Context(d.local)
    peaks = Peaks(ctx, d.local)
    fn = {"plummer1k": wl_plummer1k, "bh": wl_bh, "sph": wl_sph, "ensemble": wl_ensemble, "adjoint": wl_adjoint,
          "precision": wl_precision, "device_ics": wl_device_ics}[a.workload]
    res = {"metric": METRIC, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic",
           "workload": a.workload}
    res.update(fn(ctx, G, L, a, peaks))
    ctx.close()
    if d.rank == 0:
        print(json.dumps(res), flush=True)


def main():
    a = parse()
    d = Dist()
    try:
        if a.impl == "reference":
            run_reference(a, d)
        elif a.workload != "direct":
            run_workload(a, d)
        else:
            run_engine(a, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()

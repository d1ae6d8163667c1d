"""Benchmark: particle-steps/s of the GPU direct-sum KDK step on one GB300.

Workload (the direct-sum precision study at its largest size): Plummer sphere
N = 2^20 (reference sampler, seed 1), eps = 0.04 / N^(1/3), leapfrog KDK with
dt = 1e-4, pair forces in mixed precision (f32 pairs on f64 tile centres,
compensated sums), f64 kick/drift.  One step = one KDK step (half-kick, drift,
Hilbert sort + tile packing, all-pairs force, half-kick).  Inputs are larger
than L2 only in the f64 state, so L2 is also flushed between timed steps.

Arms:
  default          the engine (libgvs.so) on cuda:LOCAL_RANK
  --impl reference the reference's CPU algorithm (the C restatement in oracle/,
                   since the Rust reference cannot be built here) on all host
                   cores, timed on a bounded sample of the same workload.

Prints ONE JSON line on rank 0.
"""
from __future__ import annotations

import argparse
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
    ap.add_argument("--fp64-n", type=int, default=1 << 16, help="N of the bounded FP64 comparison run")
    ap.add_argument("--cpu-targets", type=int, default=1024, help="targets in the bounded CPU sample")
    ap.add_argument("--no-extras", action="store_true", help="skip FP64 / accuracy / CPU side measurements")
    ap.add_argument("--no-autotune", action="store_true", help="use the default kernel shape (profiling runs)")
    ap.add_argument("--workload", default="direct", choices=["direct", "plummer1k", "bh", "sph", "ensemble", "adjoint"],
                    help="direct (default headline); the others print their own line")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--sph-precision", default="both", choices=["both", "mixed", "f64"],
                    help="SPH workload: time both pair-arithmetic forms (and compare them), or one only")
    ap.add_argument("--nsys", type=int, default=512, help="systems in the ensemble workload")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="steps of the adjoint measurement (the adjoint workload's config is 1000)")
    ap.add_argument("--adjoint-n", type=int, default=16384, help="particles of the adjoint measurement")
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


def workload(n, seed):
    return {"workload": f"direct-sum KDK, Plummer N={n} (seed {seed}), eps=0.04/N^(1/3), dt=1e-4",
            "n": n, "seed": seed, "eps": 0.04 / n ** (1.0 / 3.0), "dt": 1e-4, "l2": "flushed between steps",
            "parallelism": "replicas (one independent system per GPU)"}


PREC = {"mixed": 3, "fp32": 2, "fp64": 1, "fp64_exact": 0}


# ---- the CPU reference arm ------------------------------------------------------------
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
    return n / step_s, cores, dt, f"{len(idx)} of {n} targets x {n} sources (one force evaluation), extrapolated"


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


def cpu_bh_sample(G, theta, eps, n=1 << 20):
    """The oracle's BarnesHut (serial build, threaded walk) for one force evaluation
    of the same two-sphere system at a bounded N."""
    import oracle as O
    q = to_oracle(G.collision(n, seed=7))
    t0 = time.perf_counter()
    O.bh(q, eps, theta)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": O.lib().orc_max_threads(), "kind": "port",
            "sample": f"one BarnesHut force evaluation (tree build + walk) of the same collision ICs at N={n}, "
                      f"theta={theta}; the step's KDK update is not included"}


def cpu_sph_sample(G, n=1 << 16):
    """The oracle's SphSolver::compute (neighbours, density, forces) once on the same
    gas sphere at a bounded N."""
    import oracle as O
    q = to_oracle(G.gas_sphere_1r(n))
    s = O.Sph()
    t0 = time.perf_counter()
    s.compute(q)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": O.lib().orc_max_threads(), "kind": "port",
            "sample": f"one SphSolver::compute of the rho~1/r sphere at N={n} (no gravity, no KDK update)"}


def run_reference(a, d: Dist):
    if d.rank != 0:
        return
    w = workload(a.n, a.seed)
    vals = []
    for _ in range(max(1, a.warmup)):
        cpu_sample(a.n, a.seed, w["eps"], max(64, a.cpu_targets // 8))
    last = None
    for s in range(a.steps):
        v, cores, secs, sample = cpu_sample(a.n, a.seed, w["eps"], a.cpu_targets, rng_seed=s)
        vals.append(v)
        last = (cores, sample)
    v = float(np.median(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": a.n / v * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (reference Plummer sampler)", "impl": "reference",
            "config": w,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": last[0], "kind": "port", "sample": last[1]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- the engine arm ---------------------------------------------------------------------
def read_traffic():
    path = os.path.join(ROOT, "profiles", "direct_mixed_traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except Exception:
        return None


def run_engine(a, d: Dist):
    import gravis_gb300 as G
    from gravis_gb300 import _lib as L
    w = workload(a.n, a.seed)
    prec = PREC[a.precision]
    ctx = G.Context(d.local)
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
    step_ms = []
    wall0 = time.perf_counter()
    with Clocks(d.local) as clk:
        for _ in range(a.steps):
            ctx.l2_flush()
            ctx.event(0)
            ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 1)
            ctx.event(1)
            step_ms.append(ctx.elapsed(0, 1))
    ctx.sync()
    wall = time.perf_counter() - wall0
    prof = ctx.profile_read()
    ctx.profile(False)
    d.barrier()
    value, t_s = replica_rate(a.n * a.steps, sum(step_ms) * 1e-3, d)
    t_ms = t_s * 1e3

    # -- e2e through the Integrator drop-in with pinned host buffers
    import torch
    names = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "mass")
    host = {k: torch.empty(a.n, dtype=torch.float64, pin_memory=True).numpy() for k in names}
    q = G.Particles(a.n)
    ctx.get_state(q)
    for k in names:
        host[k][:] = getattr(q, k)
    lib = L.load()
    ptr = {k: host[k].ctypes.data for k in names}
    e2e_s = []
    d.barrier()
    for _ in range(max(1, min(a.steps, 5))):
        t0 = time.perf_counter()
        st = lib.gvs_kdk_step_host(ctx.h, a.n, ptr["x"], ptr["y"], ptr["z"], ptr["vx"], ptr["vy"], ptr["vz"],
                                   ptr["ax"], ptr["ay"], ptr["az"], ptr["mass"], G.ALGO_DIRECT, prec, eps, 0.0, dt)
        L.check(st, ctx.h)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value, e2e_t = replica_rate(a.n * len(e2e_s), sum(e2e_s), d)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"mixed": "f32 pairs / f64 state", "fp32": "f32", "fp64": "f64",
                                           "fp64_exact": "f64"}[a.precision],
            "data": "synthetic (reference Plummer sampler, seed 1)", "config": w,
            "wall_s_timed_region": wall, "autotune": tune,
            "gpu_launches": int(prof["launches"]),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 10 * 8 * a.n,
                    "d2h_bytes_per_step": 9 * 8 * a.n, "steps": len(e2e_s)},
            "clocks": clk.summary()}

    # -- roofline of the dominant kernel (the tiled f32 pair kernel)
    kernel_ms = prof["force_ms"] / max(1, prof["force_launches"])
    flops = prof["force_flops"] / max(1, prof["force_launches"])
    peak = ctx.fp32_peak_tflops() if d.rank == 0 else None
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    tr = read_traffic()
    line["roofline"] = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                        "frac": achieved / peak if peak else None,
                        "traffic": (tr or {}).get("bytes_per_launch_scaled"),
                        "kernel": "k_direct32 (mixed, f32x2 pairs)", "kernel_ms": kernel_ms,
                        "flops_per_launch": flops, "peak_source": "measured FP32 FMA probe (gvs_measure_fp32_peak)",
                        "interactions_per_s": flops / 20.0 / (kernel_ms * 1e-3),
                        "near_field_tile_fraction": prof["near_tile_visits"] / max(1.0, prof["tile_visits"])}

    if d.rank == 0 and not a.no_extras:
        extras = {}
        # FP64 form of the same kernel, bounded N
        n64 = min(a.fp64_n, a.n)
        p64 = G.PlummerSphere(n64, seed=a.seed).generate()
        e64 = 0.04 / n64 ** (1.0 / 3.0)
        rates = {}
        for name, pr in (("fp64", 1), ("mixed", 3)):
            ctx.set_state(p64)
            ctx.compute_forces(G.ALGO_DIRECT, pr, e64)
            ctx.profile(True)
            for _ in range(3):
                ctx.compute_forces(G.ALGO_DIRECT, pr, e64)
            pf = ctx.profile_read()
            ctx.profile(False)
            rates[name] = pf["force_flops"] / 20.0 / (pf["force_ms"] * 1e-3)
        extras["fp64_interactions_per_s"] = rates["fp64"]
        extras["mixed_interactions_per_s_same_n"] = rates["mixed"]
        extras["mixed_vs_fp64"] = rates["mixed"] / rates["fp64"]
        extras["fp64_n"] = n64
        # force error of mixed at the bench N against exact f64 on a target subset
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, 3, eps)
        full = G.Particles(a.n)
        ctx.get_state(full)
        idx = np.sort(np.random.default_rng(123).choice(a.n, size=1024, replace=False))
        ref = ctx.direct_subset(idx, eps, G.PREC_FP64_EXACT)
        got = full.acc()[idx]
        extras["force_rel_rms_mixed_vs_fp64"] = float(np.sqrt(((got - ref) ** 2).sum() / (ref ** 2).sum()))
        extras["force_rel_err_subset"] = "1024 random targets, exact f64 reference on the GPU"
        extras["adjoint"] = adjoint_ratio(ctx, G, n=a.adjoint_n, steps=a.adjoint_steps, every=100)
        line["extras"] = extras
        try:
            v, cores, secs, sample = cpu_sample(a.n, a.seed, eps, a.cpu_targets)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                                    "seconds": secs}
        except Exception as ex:  # the oracle must be built (build() does it)
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": None, "kind": "port",
                                    "sample": f"unavailable: {ex}"}
    ctx.close()
    if d.rank == 0:
        print(json.dumps(line), flush=True)


def adjoint_ratio(ctx, G, n=16384, steps=200, every=100, seed=42, eps=0.01, dt=1e-3, check_fp64=True):
    """Adjoint workload: L = sum m |x(T) - x*|^2 for a Plummer sphere; cost of the
    backward sweep over the cost of the plain forward run, and the relative error
    of the mixed-precision gradient against the f64 adjoint."""
    p = G.PlummerSphere(n, seed=seed).generate()
    rng = np.random.default_rng(seed)

    def run(prec):
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
        xstar = x + 0.01 * np.random.default_rng(seed + 1).standard_normal(x.shape)
        ctx.event(6)
        g = ctx.adjoint_backward(2.0 * p.mass[:, None] * (x - xstar))
        ctx.event(7)
        return fwd_plain, fwd_ck, ctx.elapsed(6, 7), g

    f_plain, f_ck, bwd, g = run(G.PREC_MIXED)
    out = {"workload": f"Plummer N={n} seed {seed}, eps={eps}, dt={dt}, {steps} steps, f64 checkpoints every {every}",
           "forward_ms": f_plain, "forward_with_checkpoints_ms": f_ck, "backward_ms": bwd,
           "adjoint_over_forward": bwd / f_plain}
    if check_fp64:
        _, _, bwd64, g64 = run(G.PREC_FP64)
        out["grad_rel_err_mixed_vs_fp64_adjoint"] = {
            k: float(np.linalg.norm(g[k] - g64[k]) / np.linalg.norm(g64[k])) for k in ("x", "v", "m")}
        out["fp64_backward_ms"] = bwd64
    del rng
    return out


def hbm_peak_gbs():
    """HBM copy bandwidth measured on this machine (MEASURED_PEAKS.json beside this file), else
    the fallback figure of one earlier GB300 measurement; returns (GB/s, source)."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def run_workload(a, d):
    """Secondary workloads (one JSON line each; the default run is the direct sum)."""
    import gravis_gb300 as G
    ctx = G.Context(d.local)
    res = {"metric": METRIC, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic"}
    if a.workload == "bh":
        n = a.n
        p = G.collision(n, seed=7)
        eps, theta, dt = 1e-3, a.theta, 5e-4
        prec = G.PREC_FP32 if a.precision in ("mixed", "fp32") else G.PREC_FP64
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_BH, prec, eps, theta)
        for _ in range(a.warmup):
            ctx.kdk_steps(G.ALGO_BH, prec, eps, theta, dt, 1)
        ctx.profile(True)
        ms = []
        with Clocks(d.local) as clk:
            for _ in range(a.steps):
                ctx.l2_flush()
                ctx.event(0)
                ctx.kdk_steps(G.ALGO_BH, prec, eps, theta, dt, 1)
                ctx.event(1)
                ms.append(ctx.elapsed(0, 1))
        prof = ctx.profile_read()
        ctx.profile(False)
        t = sum(ms)
        idx = np.sort(np.random.default_rng(1).choice(n, 4096, replace=False))
        ref = ctx.direct_subset(idx, eps)
        q = G.Particles(n)
        ctx.get_state(q)
        ctx.compute_forces(G.ALGO_BH, prec, eps, theta)
        ctx.get_state(q)
        rel = np.sqrt((((q.acc()[idx] - ref) ** 2).sum(1) / (ref ** 2).sum(1)).mean())
        # the walk forms side by side on the final state: time and distance to the f64 walk
        # (fp32: the group walk at its automatic group size, the FP32 default;
        # fp32_groupG: G-particle groups; fp32_per_particle: the reference's
        # per-particle test on f32 positions)
        walks = {}
        for wname, wp, grp in (("fp64", G.PREC_FP64, -1), ("mixed", G.PREC_MIXED, -1), ("fp32", G.PREC_FP32, -1),
                               ("fp32_group32", G.PREC_FP32, 32), ("fp32_group64", G.PREC_FP32, 64),
                               ("fp32_group128", G.PREC_FP32, 128), ("fp32_per_particle", G.PREC_FP32, 0)):
            ctx.set_bh_walk(grp)
            ctx.compute_forces(G.ALGO_BH, wp, eps, theta)  # builds the packed node arrays
            ctx.profile(True)
            ctx.compute_forces(G.ALGO_BH, wp, eps, theta)
            pw = ctx.profile_read()
            ctx.profile(False)
            qw = G.Particles(n)
            ctx.get_state(qw)
            walks[wname] = {"walk_ms": pw["force_ms"], "acc": qw.acc()}
            if pw["bh_groups"]:
                walks[wname].update({"groups": pw["bh_groups"], "groups_walked_per_particle": pw["bh_group_fallbacks"],
                                     "group_iterations": pw["bh_group_iterations"],
                                     "interactions_per_particle": pw["bh_group_interactions"] / n,
                                     "interactions_per_s": pw["bh_group_interactions"] / (pw["force_ms"] * 1e-3)})
        ctx.set_bh_walk(-1)
        a64 = walks["fp64"]["acc"]
        for wname in walks:
            aw = walks[wname].pop("acc")
            if wname != "fp64":
                walks[wname]["rel_rms_vs_fp64_walk"] = float(np.sqrt(((aw - a64) ** 2).sum() / (a64 ** 2).sum()))
            walks[wname]["per_particle_rms_rel_err_vs_exact_f64_direct"] = float(
                np.sqrt((((aw[idx] - ref) ** 2).sum(1) / (ref ** 2).sum(1)).mean()))
        # roofline of the walk: counted node/particle terms x 20 flop against the FP32 peak
        walk_s = prof["force_ms"] * 1e-3
        terms_s = prof["bh_group_interactions"] / walk_s if walk_s > 0 else 0.0
        peak32 = ctx.fp32_peak_tflops()
        res["roofline"] = {"bound": "fp32", "achieved": terms_s * 20 / 1e12, "peak": peak32, "unit": "TFLOP/s",
                           "frac": terms_s * 20 / 1e12 / peak32 if peak32 else None, "traffic": None,
                           "kernel": "k_walk_group (FP32 group walk)",
                           "terms_per_s": terms_s, "terms_per_particle": prof["bh_group_interactions"] / (n * a.steps),
                           "peak_source": "measured FP32 FMA probe (gvs_measure_fp32_peak)",
                           "work_unit": "20 flop per node or particle term evaluated for a real particle; "
                                        "DRAM traffic of the walk is in profiles/ (ncu)"}
        res.update({"value": n * a.steps / (t * 1e-3), "ms_per_step": t / a.steps, "dtype": "f32 walk / f64 state",
                    "walk_forms": walks,
                    "config": {"workload": f"Barnes-Hut KDK, two Plummer spheres N={n} seed 7, theta={theta}, "
                                           f"eps={eps}, dt={dt}", "n": n, "theta": theta},
                    "walk_ms_per_step": prof["force_ms"] / max(1, prof["force_launches"]),
                    "gpu_launches": int(prof["launches"]),
                    "accuracy": {"per_particle_rms_rel_err_vs_exact_f64_direct": float(rel),
                                 "subset": "4096 random particles"},
                    "clocks": clk.summary()})
        if d.rank == 0 and not a.no_extras:
            res["cpu_baseline"] = cpu_bh_sample(G, theta, eps)
    elif a.workload == "sph":
        n = a.n
        p = G.gas_sphere_1r(n)
        eps = 0.3 * (4.0 / 3.0 * np.pi / n) ** (1.0 / 3.0)
        theta = a.theta
        sph = G.SphSolver(ctx)
        import ctypes as C
        gas_fields = ("density", "pressure", "internal_energy", "du_dt", "smoothing_length", "sound_speed",
                      "alpha_visc")

        def upload():
            ctx.set_state(p)
            ctx._ck(ctx._lib.gvs_set_gas(ctx.h, *(G.engine._ptr(getattr(p, f)) for f in gas_fields)))

        def sph_only(prec):
            """one SphSolver::compute on the initial state, SPH terms only"""
            upload()
            sph.params.precision = prec
            ctx._ck(ctx._lib.gvs_sph_compute(ctx.h, C.byref(sph.params), None, None, None, None))
            q = G.Particles(n)
            ctx.get_state(q)
            ctx.get_gas(q)
            return q

        def timed(prec):
            upload()
            sph.params.precision = prec
            ctx.compute_forces(G.ALGO_BH, G.PREC_FP32, eps, theta)
            ctx._ck(ctx._lib.gvs_sph_compute(ctx.h, C.byref(sph.params), None, None, None, None))
            dtc = C.c_double()
            ctx._ck(ctx._lib.gvs_sph_timestep(ctx.h, C.byref(sph.params), C.byref(dtc)))
            dt = dtc.value

            def step(dt):
                ctx._ck(ctx._lib.gvs_sph_step(ctx.h, C.byref(sph.params), G.ALGO_BH, G.PREC_FP32, eps, theta, dt,
                                              C.byref(dtc)))
                return min(dtc.value, 1.5 * dt)

            for _ in range(a.warmup):
                dt = step(dt)
            ms = []
            with Clocks(d.local) as clk:
                for _ in range(a.steps):
                    ctx.l2_flush()
                    ctx.event(0)
                    dt = step(dt)
                    ctx.event(1)
                    ms.append(ctx.elapsed(0, 1))
            return sum(ms), clk.summary()

        if a.sph_precision != "both":  # one form only (profiling runs): no comparison
            prec = G.PREC_MIXED if a.sph_precision == "mixed" else G.PREC_FP64_EXACT
            t, clk = timed(prec)
            res.update({"value": n * a.steps / (t * 1e-3), "ms_per_step": t / a.steps,
                        "dtype": "f32 SPH pair terms (mixed)" if prec == G.PREC_MIXED else "f64 SPH",
                        "config": {"workload": f"grad-h SPH + BH gravity, rho~1/r gas sphere N={n}, "
                                               f"{a.sph_precision} pair arithmetic only", "n": n},
                        "clocks": clk})
            ctx.close()
            if d.rank == 0:
                print(json.dumps(res), flush=True)
            return
        qe = sph_only(G.PREC_FP64_EXACT)
        ctx.profile(True)
        qm = sph_only(G.PREC_MIXED)
        redo = ctx.profile_read()["sph_f64_redo"]
        ctx.profile(False)

        def rel(f):
            x, y = getattr(qm, f), getattr(qe, f)
            return float(np.sqrt(((x - y) ** 2).sum() / max((y ** 2).sum(), 1e-300)))

        errs = {f: rel(f) for f in ("density", "smoothing_length", "ax", "ay", "az", "du_dt")}
        # where the relative RMS comes from: particles whose h differs by more than 1e-5 are
        # those whose h-iteration stopping decision (|dh|/h < 1e-3) fell the other way
        dh = np.abs(qm.smoothing_length - qe.smoothing_length) / np.maximum(qe.smoothing_length, 1e-300)
        am, ae = np.stack([qm.ax, qm.ay, qm.az], 1), np.stack([qe.ax, qe.ay, qe.az], 1)
        scale = np.sqrt((ae ** 2).sum(1).mean())
        ea = np.sqrt(((am - ae) ** 2).sum(1)) / scale
        errs["h_iteration_outliers"] = int((dh > 1e-5).sum())
        errs["particles_rerun_in_f64"] = int(redo)
        errs["per_particle_a_err_over_rms_a"] = {"p50": float(np.percentile(ea, 50)),
                                                 "p99": float(np.percentile(ea, 99)),
                                                 "p99.9": float(np.percentile(ea, 99.9)),
                                                 "max": float(ea.max())}
        t_ex, _ = timed(G.PREC_FP64_EXACT)
        t, clk = timed(G.PREC_MIXED)
        res.update({"value": n * a.steps / (t * 1e-3), "ms_per_step": t / a.steps,
                    "dtype": "f32 SPH pair terms (mixed) / f64 state / f32 BH walk",
                    "config": {"workload": f"grad-h SPH + BH gravity, rho~1/r gas sphere N={n}, u=0.05, "
                                           f"Wendland C2, eta=1.2, theta={theta}, eps={eps:.3g}, CFL 0.3",
                               "n": n},
                    "f64_exact": {"value": n * a.steps / (t_ex * 1e-3), "ms_per_step": t_ex / a.steps,
                                  "what": "the same steps with the reference's f64 SPH arithmetic"},
                    "mixed_over_f64": t_ex / t,
                    "mixed_vs_f64_rel_rms": errs, "clocks": clk})
        # roofline per the algorithmic bytes of one SPH step (density 120 B, forces 160 B,
        # neighbour rows 840 B, KDK 120 B per particle)
        hbm, hbm_src = hbm_peak_gbs()
        gbs = n * 1240.0 / (t / a.steps * 1e-3) / 1e9
        res["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                           "traffic": None, "bytes_per_particle_step": 1240, "peak_source": hbm_src,
                           "note": "the SPH kernels are issue- and latency-bound well below this roofline "
                                   "(neighbour walk, f32 pair gathers); their ncu figures are in profiles/"}
        if d.rank == 0 and not a.no_extras:
            res["cpu_baseline"] = cpu_sph_sample(G)
    elif a.workload == "ensemble":
        from gravis_gb300.engine import plummer_ensemble
        sizes = G.ensemble_sizes(a.nsys, seed=2024)
        p = plummer_ensemble(sizes)
        n, eps, dt = p.count, 0.01, 1e-3
        ctx.set_state(p)
        ctx.ensemble_setup(sizes, eps)
        ctx.ensemble_forces()
        ctx.ensemble_kdk_steps(dt, max(1, a.warmup), True)
        ctx.sync()
        ctx.event(0)
        ctx.ensemble_kdk_steps(dt, a.steps, True)
        ctx.event(1)
        t = ctx.elapsed(0, 1)
        # the same systems, one single-system context each, stepped one after another
        ctxs, subs, o = [], [], 0
        for m in sizes:
            q = G.Particles(int(m))
            for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
                getattr(q, f)[:] = getattr(p, f)[o:o + m]
            o += m
            c = G.Context(d.local)
            c.set_state(q)
            c.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
            ctxs.append(c)
        for c in ctxs:
            c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 1)
        for c in ctxs:
            c.sync()
        # (a) every step, every system in turn, one step per call
        kb = 2
        t0 = time.perf_counter()
        for _ in range(kb):
            for c in ctxs:
                c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 1)
        for c in ctxs:
            c.sync()
        tb = (time.perf_counter() - t0) * 1e3
        # (b) each system all its steps in one call (its step replayed as a CUDA graph);
        #     the contexts' streams are independent, so systems may overlap on the GPU
        for c in ctxs:
            c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 2)  # capture
        for c in ctxs:
            c.sync()
        kg = max(2, min(a.steps, 10))
        t0 = time.perf_counter()
        for c in ctxs:
            c.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, kg)
        for c in ctxs:
            c.sync()
        tg = (time.perf_counter() - t0) * 1e3
        for c in ctxs:
            c.close()
        v = n * a.steps / (t * 1e-3)
        vb = n * kb / (tb * 1e-3)
        vg = n * kg / (tg * 1e-3)
        best = max(vb, vg)
        res.update({"value": v, "ms_per_step": t / a.steps, "dtype": "f32 pairs / f64 state",
                    "config": {"workload": f"{a.nsys} Plummer systems, N_i log-uniform [256, 16384] (seed 2024), "
                                           f"seeds 1000+i, eps={eps}, dt={dt}, CUDA-graph steps",
                               "n_total": n, "sum_n2": float((sizes.astype(np.float64) ** 2).sum())},
                    "separate_systems": {"value": vb, "ms_per_step": tb / kb,
                                         "how": "one single-system context per system, each step all systems in turn"},
                    "separate_systems_graphs": {"value": vg, "ms_per_step": tg / kg,
                                                "how": "one context per system, each runs its steps as CUDA-graph "
                                                       "replays on its own stream, systems launched in turn"},
                    "batched_over_separate_per_step_calls": v / vb,
                    "batched_over_separate_graphs": v / vg,
                    "batched_over_separate": v / best})
    elif a.workload == "plummer1k":
        # the headless plummer run: N=1000, seed 42, eps=0.01, dt=1e-3; a step is one KDK step
        n, eps, dt = 1000, 0.01, 1e-3
        steps = max(a.steps, 100)
        p = G.PlummerSphere(n, seed=42).generate()
        out = {}
        for name, prec in (("fp64_exact", G.PREC_FP64_EXACT), ("mixed", G.PREC_MIXED)):
            ctx.set_state(p)
            ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
            e0 = ctx.diagnostics(eps).total_energy
            ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, max(2, a.warmup))  # warm, captures the step graph
            ctx.sync()
            ctx.event(0)
            ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, steps)
            ctx.event(1)
            t = ctx.elapsed(0, 1)
            e1 = ctx.diagnostics(eps).total_energy
            out[name] = {"value": n * steps / (t * 1e-3), "ms_per_step": t / steps,
                         "rel_energy_drift": abs((e1 - e0) / e0), "steps": steps + max(2, a.warmup)}
        # the reference's CPU path on the host cores: a bounded run of the same steps
        import oracle as O
        q = O.plummer(n, 42)
        g = O.gravity(O.GRAV_BF, eps)
        O.bf_serial(q, eps)
        ks = 50
        t0 = time.perf_counter()
        O.kdk_steps(q, g, dt, ks)
        tc = time.perf_counter() - t0
        res.update({"value": out["mixed"]["value"], "ms_per_step": out["mixed"]["ms_per_step"],
                    "dtype": "f32 pairs / f64 state", "steps": steps,
                    "config": {"workload": f"headless plummer: N={n} seed 42, eps={eps}, dt={dt}, {steps} KDK steps "
                                           "per timed run, each step a CUDA-graph replay", "n": n},
                    "fp64_exact": out["fp64_exact"], "mixed": out["mixed"],
                    "cpu_baseline": {"value": n * ks / tc, "unit": UNIT, "cores": 1, "kind": "port",
                                     "sample": f"{ks} KDK steps of the same system, serial symmetric BruteForce"}})
    elif a.workload == "adjoint":
        r = adjoint_ratio(ctx, G, n=a.adjoint_n, steps=a.adjoint_steps, every=100)
        res.update({"value": r["adjoint_over_forward"], "unit": "backward/forward", "higher_is_better": False,
                    "adjoint": r})
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

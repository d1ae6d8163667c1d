"""Every engine path on small cases, run against the bounds-checked library
(libgvs_checked.so, loaded when GVS_CHECKED=1 is set before the first load).

Used by tests/test_checked_gpu.py in a child process: each step compares the
result with the oracle (or with the normal path's own invariant) and reads the
device error word, which must stay zero -- no index any kernel computed fell
outside its array and the tree kept its invariants.  Prints one JSON line.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import gravis_gb300 as G  # noqa: E402
import oracle as O  # noqa: E402
from gravis_gb300 import _lib as L  # noqa: E402


def to_oracle(p):
    q = O.Particles(p.count)
    for a, b in (("x", "x"), ("y", "y"), ("z", "z"), ("vx", "vx"), ("vy", "vy"), ("vz", "vz"), ("mass", "mass"),
                 ("density", "density"), ("pressure", "pressure"), ("internal_energy", "u"),
                 ("smoothing_length", "h"), ("sound_speed", "cs"), ("alpha_visc", "alpha"),
                 ("particle_type", "ptype")):
        getattr(q, b)[:] = getattr(p, a)
    return q


def rel(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def main():
    assert os.environ.get("GVS_CHECKED") == "1"
    version = L.load().gvs_version().decode()
    out = {"version": version, "steps": {}}
    ctx = G.Context(0)

    def step(name, err=None, bar=None):
        flags = ctx.device_errors()
        out["steps"][name] = {"flags": flags, "err": err, "bar": bar}

    # direct sum, every precision, against the oracle
    for n in (1000, 4097):
        p = G.PlummerSphere(n, seed=3).generate()
        q = O.plummer(n, 3)
        eps = 0.01
        O.bf_serial(q, eps)
        for name, prec, bar in (("exact", G.PREC_FP64_EXACT, 0.0), ("fp64", G.PREC_FP64, 1e-12),
                                ("fp32", G.PREC_FP32, 1e-4), ("mixed", G.PREC_MIXED, 1e-6)):
            a = p.copy()
            a.clear_accelerations()
            G.BruteForce(eps, prec, ctx).compute_accelerations(a)
            step(f"direct_{name}_{n}", rel(a.acc(), q.acc()), bar)
    # KDK steps (graph replay) and the one-launch tiny path
    for n, prec in ((1000, G.PREC_MIXED), (1000, G.PREC_FP64_EXACT), (5, G.PREC_FP64_EXACT)):
        p = G.PlummerSphere(n, seed=5).generate()
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, 0.02)
        ctx.kdk_steps(G.ALGO_DIRECT, prec, 0.02, 0.0, 1e-3, 20)
        q = O.plummer(n, 5)
        O.bf_serial(q, 0.02)
        O.kdk_steps(q, O.gravity(O.GRAV_BF, 0.02), 1e-3, 20)
        r = G.Particles(n)
        ctx.get_state(r)
        step(f"kdk_{prec}_{n}", rel(r.x, q.x), 0.0 if prec == G.PREC_FP64_EXACT else 1e-9)
    # octree and Barnes-Hut walks
    p = G.collision(4096, seed=7)
    ctx.set_state(p)
    t = ctx.tree_export()
    ref = O.octree_leaves(to_oracle(p))
    step("tree_export", float(t["nnodes"] != ref["nnodes"]), 0.0)
    q = to_oracle(p)
    O.bh(q, 0.05, 0.5)
    for name, prec, bar in (("f64", G.PREC_FP64, 1e-12), ("mixed", G.PREC_MIXED, 1e-6), ("group", G.PREC_FP32, 1e-2)):
        a = p.copy()
        a.clear_accelerations()
        G.BarnesHut(0.05, 0.5, prec, ctx).compute_accelerations(a)
        step(f"bh_{name}", rel(a.acc(), q.acc()), bar)
    ctx.set_bh_walk(0)
    a = p.copy()
    a.clear_accelerations()
    G.BarnesHut(0.05, 0.5, G.PREC_FP32, ctx).compute_accelerations(a)
    ctx.set_bh_walk(-1)
    step("bh_f32_per_particle", rel(a.acc(), q.acc()), 1e-2)
    # SPH, both arithmetic forms, and a step
    g = G.gas_sphere_1r(4000)
    g.vx[:] = -0.1 * g.x
    q = to_oracle(g)
    s = O.Sph()
    s.compute(q)
    for name, prec, bar in (("f64", G.PREC_FP64_EXACT, 1e-10), ("mixed", G.PREC_MIXED, 1e-6)):
        a = g.copy()
        sph = G.SphSolver(ctx)
        sph.params.precision = prec
        sph.compute(a)
        step(f"sph_{name}", max(rel(a.ax, q.ax), rel(a.density, q.density)), bar)
    a = g.copy()
    sph = G.SphSolver(ctx)
    G.step_with_sph(a, G.BarnesHut(0.01, 0.5, G.PREC_FP32, ctx), sph, 1e-4)
    step("sph_step", float(not np.isfinite(a.x).all()), 0.0)
    # ensemble against single-system runs
    sizes = np.array([100, 333, 1000, 2500], dtype=np.int64)
    from gravis_gb300.engine import plummer_ensemble
    pe = plummer_ensemble(sizes)
    ctx.set_state(pe)
    ctx.ensemble_setup(sizes, 0.01)
    ctx.ensemble_forces()
    r = G.Particles(pe.count)
    ctx.get_state(r)
    worst, o = 0.0, 0
    for m in sizes:
        sub = G.Particles(int(m))
        for f in ("x", "y", "z", "mass"):
            getattr(sub, f)[:] = getattr(pe, f)[o:o + m]
        qq = to_oracle(sub)
        O.bf_serial(qq, 0.01)
        worst = max(worst, rel(r.acc()[o:o + m], qq.acc()))
        o += m
    step("ensemble", worst, 1e-6)
    ctx.ensemble_kdk_steps(1e-3, 3, True)
    step("ensemble_steps", None, None)
    # adjoint, both precisions
    p = G.PlummerSphere(256, seed=4).generate()
    grads = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        ctx.set_state(p)
        ctx.adjoint_forward(prec, 0.05, 1e-3, 20, 10)
        grads[prec] = ctx.adjoint_backward(np.ones((256, 3)))
    step("adjoint", rel(grads[G.PREC_MIXED]["x"], grads[G.PREC_FP64]["x"]), 1e-4)
    # diagnostics
    p = G.PlummerSphere(3000, seed=8).generate()
    ctx.set_state(p)
    d = ctx.diagnostics(0.03)
    e = O.diagnostics(O.plummer(3000, 8), 0.03)
    step("diagnostics", abs(d.potential_energy - e["potential_energy"]) / abs(e["potential_energy"]), 1e-12)
    ctx.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()

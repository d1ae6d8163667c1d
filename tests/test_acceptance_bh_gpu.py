"""The reference's Barnes-Hut integration tests (crates/sim-core/tests/barnes_hut.rs), run on
the GPU walks with the same scenarios, seeds, softenings, timesteps, durations and bars:
the f64 walk (the reference's arithmetic) and the mixed walk (the reference's decisions,
f32 terms on float-float separations).

  force_accuracy_theta_05 / _03   (:52-72)  RMS relative force error against BruteForce
  force_accuracy_monotonic        (:74-101) the error grows with theta
  virial_equilibrium_plummer_bh   (:142-193) N = 500, 10 t_dyn, virial ratio and energy
and determinism.rs (both solvers, twice, bit for bit) and the cold collapse of galaxy.rs
(energy with BarnesHut; its IC properties are checked on the CPU in test_abi_cpu.py).

energy_conservation_kepler_bh (:103-140) is left out: on two bodies the walk opens the root
and sums the single pair exactly (the Kepler tests of the direct sum cover that orbit), and
its 10^6 steps would each rebuild a tree.
"""
import numpy as np
import pytest

import gravis_gb300 as G

pytestmark = pytest.mark.gpu

WALKS = [G.PREC_FP64, G.PREC_MIXED]


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def rms_force_error(ctx, n, theta, softening, prec):
    """barnes_hut.rs:12-48: sqrt(mean_i |a_BH - a_BF|^2 / |a_BF|^2), particles with
    |a_BF|^2 < 1e-30 skipped in the sum but not in the mean."""
    p = G.PlummerSphere(n, seed=42).generate()
    bf = p.copy()
    bf.clear_accelerations()
    G.BruteForce(softening, G.PREC_FP64_EXACT, ctx).compute_accelerations(bf)
    bh = p.copy()
    bh.clear_accelerations()
    G.BarnesHut(softening, theta, prec, ctx).compute_accelerations(bh)
    a_bf, a_bh = bf.acc(), bh.acc()
    mag2 = (a_bf ** 2).sum(1)
    keep = mag2 >= 1e-30
    err2 = ((a_bh - a_bf) ** 2).sum(1)
    return float(np.sqrt((err2[keep] / mag2[keep]).sum() / n))


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_force_accuracy_theta_05(ctx, prec):
    err = rms_force_error(ctx, 1000, 0.5, 0.05, prec)
    print(f"RMS force error at theta=0.5: {err:.6e}")
    assert err < 0.01


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_force_accuracy_theta_03(ctx, prec):
    err = rms_force_error(ctx, 1000, 0.3, 0.05, prec)
    print(f"RMS force error at theta=0.3: {err:.6e}")
    assert err < 0.005


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_force_accuracy_monotonic_with_theta(ctx, prec):
    thetas = [0.3, 0.5, 0.7, 1.0]
    errors = [rms_force_error(ctx, 500, t, 0.05, prec) for t in thetas]
    print("force accuracy sweep: " + ", ".join(f"theta={t}: {e:.3e}" for t, e in zip(thetas, errors)))
    for i in range(1, len(errors)):
        assert errors[i] >= errors[i - 1] * 0.5


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_virial_equilibrium_plummer_bh(ctx, prec):
    sc = G.PlummerSphere(500, seed=42)
    p = sc.generate()
    dt, eps = sc.suggested_dt(), sc.suggested_softening()
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_BH, prec, eps, 0.5)
    e0 = ctx.diagnostics(eps).total_energy
    steps = int(round(10.0 * 1.0 / dt))
    worst = 0.0
    done = 0
    while done < steps:
        k = min(100, steps - done)
        ctx.kdk_steps(G.ALGO_BH, prec, eps, 0.5, dt, k)
        done += k
        if done % 100 == 0:
            worst = max(worst, abs(ctx.diagnostics(eps).virial_ratio - 1.0))
    de = abs((ctx.diagnostics(eps).total_energy - e0) / abs(e0))
    print(f"Plummer BH virial max deviation {worst:.4f}, dE/E {de:.3e}")
    assert worst < 0.5
    assert de < 0.01


# ---- determinism.rs and galaxy.rs (the cold collapse) --------------------------------
def run_sim(p, algo, prec, eps, theta, dt, steps):
    """determinism.rs:12-27 in a fresh context: forces, then `steps` KDK steps."""
    c = G.Context(0)
    try:
        c.set_state(p)
        c.compute_forces(algo, prec, eps, theta)
        c.kdk_steps(algo, prec, eps, theta, dt, steps)
        q = G.Particles(p.count)
        c.get_state(q)
    finally:
        c.close()
    return np.stack([q.x, q.y, q.z], 1)


@pytest.mark.parametrize("algo,prec", [(G.ALGO_DIRECT, G.PREC_FP64_EXACT), (G.ALGO_DIRECT, G.PREC_MIXED),
                                       (G.ALGO_BH, G.PREC_FP64), (G.ALGO_BH, G.PREC_MIXED),
                                       (G.ALGO_BH, G.PREC_FP32)],
                         ids=["bf-exact", "bf-mixed", "bh-f64", "bh-mixed", "bh-f32"])
def test_deterministic(algo, prec):
    """determinism.rs:29-69: N = 200 seed 42, eps 0.05, dt 1e-3, 50 steps, twice: the same
    positions bit for bit."""
    p = G.PlummerSphere(200, seed=42).generate()
    a = run_sim(p, algo, prec, 0.05, 0.5, 1e-3, 50)
    b = run_sim(p, algo, prec, 0.05, 0.5, 1e-3, 50)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_cold_collapse_energy_conservation(ctx, prec):
    """galaxy.rs:58-89: ColdCollapse N = 500, suggested eps and dt, BarnesHut theta 0.5,
    100 steps: |dE/E| < 5 %."""
    sc = G.ColdCollapse(500)
    p = sc.generate()
    eps, dt = sc.suggested_softening(), sc.suggested_dt()
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_BH, prec, eps, 0.5)
    e0 = ctx.diagnostics(eps).total_energy
    ctx.kdk_steps(G.ALGO_BH, prec, eps, 0.5, dt, 100)
    drift = abs((ctx.diagnostics(eps).total_energy - e0) / e0)
    print(f"cold collapse dE/E over 100 steps {drift:.3e}")
    assert drift < 0.05


@pytest.mark.parametrize("prec", WALKS, ids=["f64", "mixed"])
def test_barnes_hut_scaling_is_nlogn(ctx, prec):
    """scaling.rs:14-80 with the walk's summed terms in place of wall time (a GPU at
    N <= 20000 is bound by launch latency, not by the walk's work): Plummer seed 42,
    theta 0.5, eps 0.05, N = 2^14 ... 2^18; the log-log slope of the work over the last
    four sizes lies in [0.8, 1.8] (N log N, not N^2)."""
    ns = [1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18]
    work = []
    for n in ns:
        p = G.PlummerSphere(n, seed=42).generate()
        p.clear_accelerations()
        try:
            ctx.profile(True)
            G.BarnesHut(0.05, 0.5, prec, ctx).compute_accelerations(p)
            work.append(ctx.profile_read()["bh_walk_terms"])
        finally:
            ctx.profile(False)
    x, y = np.log(ns[1:]), np.log(work[1:])
    slope = float(((x - x.mean()) * (y - y.mean())).sum() / ((x - x.mean()) ** 2).sum())
    print("terms: " + ", ".join(f"N={n}: {w}" for n, w in zip(ns, work)) + f"; log-log slope {slope:.3f}")
    assert 0.8 <= slope <= 1.8

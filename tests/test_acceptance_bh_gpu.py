"""The reference's Barnes-Hut integration tests (crates/sim-core/tests/barnes_hut.rs), run on
the GPU walks with the same scenarios, seeds, softenings, timesteps, durations and bars:
the f64 walk (the reference's arithmetic) and the mixed walk (the reference's decisions,
f32 terms on float-float separations).

  force_accuracy_theta_05 / _03   (:52-72)  RMS relative force error against BruteForce
  force_accuracy_monotonic        (:74-101) the error grows with theta
  virial_equilibrium_plummer_bh   (:142-193) N = 500, 10 t_dyn, virial ratio and energy

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

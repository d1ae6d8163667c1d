"""GPU parity of the direct sum, KDK and diagnostics against the oracle.

Bars: FP64_EXACT is bit-identical to the reference arithmetic (integer-like
bar); FP64 (tiled, FMA) within 1e-13 relative RMS; MIXED within 1e-6 relative
RMS (the precision target of the mixed form); FP32 within 1e-4.  Relative RMS is
sqrt(sum |a - a_ref|^2 / sum |a_ref|^2).
"""
import numpy as np
import pytest

import gravis_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def rel_rms(a, ref):
    return float(np.sqrt(((a - ref) ** 2).sum() / (ref ** 2).sum()))


def gpu_acc(ctx, p, eps, prec):
    q = p.copy()
    q.clear_accelerations()
    G.BruteForce(eps, prec, ctx).compute_accelerations(q)
    return q.acc()


def oracle_acc(p_or, eps):
    q = p_or.copy()
    q.clear_accelerations()
    O.bf_gather(q, eps)
    return q.acc()


@pytest.mark.parametrize("n", [1, 2, 3, 31, 127, 128, 129, 1000, 4097])
def test_exact_bitwise(ctx, n):
    p = G.PlummerSphere(n, seed=n).generate()
    q = O.plummer(n, n)
    eps = 0.01
    a = gpu_acc(ctx, p, eps, G.PREC_FP64_EXACT)
    q.clear_accelerations()
    O.bf_serial(q, eps)
    assert np.array_equal(a, q.acc())


def test_exact_force_quarter(ctx):
    """gravity.rs:107-120 on the GPU: a = 0.25 at r = 2 with eps = 0."""
    p = G.Particles(2)
    p.x[1] = 2.0
    p.mass[:] = 1.0
    for prec in (G.PREC_FP64_EXACT, G.PREC_FP64, G.PREC_MIXED, G.PREC_FP32):
        a = gpu_acc(ctx, p, 0.0, prec)
        assert abs(a[0, 0] - 0.25) < 1e-6 and abs(a[0, 0] + a[1, 0]) < 1e-6, (prec, a)
        assert np.all(np.isfinite(a))


def test_accumulate_semantics(ctx):
    """compute_accelerations adds onto whatever ax..az hold (gravity.rs:6-10)."""
    p = G.PlummerSphere(300, seed=5).generate()
    for prec in (G.PREC_FP64_EXACT, G.PREC_MIXED):
        base = gpu_acc(ctx, p, 0.02, prec)
        q = p.copy()
        q.ax[:], q.ay[:], q.az[:] = 1.0, -2.0, 3.0
        G.BruteForce(0.02, prec, ctx).compute_accelerations(q)
        assert np.allclose(q.acc() - np.array([1.0, -2.0, 3.0]), base, rtol=0, atol=1e-12)


@pytest.mark.parametrize("n", [1000, 16384, 65537])
def test_precisions_vs_oracle(ctx, n):
    p = G.PlummerSphere(n, seed=3).generate()
    eps = 0.04 / n ** (1.0 / 3.0)
    ref = oracle_acc(O.plummer(n, 3), eps)
    e64 = rel_rms(gpu_acc(ctx, p, eps, G.PREC_FP64), ref)
    emx = rel_rms(gpu_acc(ctx, p, eps, G.PREC_MIXED), ref)
    e32 = rel_rms(gpu_acc(ctx, p, eps, G.PREC_FP32), ref)
    print(f"n={n} rel RMS fp64={e64:.2e} mixed={emx:.2e} fp32={e32:.2e}")
    assert e64 < 1e-13
    assert emx <= 1e-6
    assert e32 <= 1e-4
    assert emx < e32


def test_mixed_deterministic(ctx):
    p = G.PlummerSphere(20000, seed=11).generate()
    a = gpu_acc(ctx, p, 0.001, G.PREC_MIXED)
    b = gpu_acc(ctx, p, 0.001, G.PREC_MIXED)
    assert np.array_equal(a, b)


def test_kdk_trajectory_bitwise(ctx):
    """50 KDK steps (integrator.rs:42-76) with exact f64 forces equal the oracle bit for bit."""
    n, eps, dt = 200, 0.05, 1e-3
    p = G.PlummerSphere(n, seed=42).generate()
    q = O.plummer(n, 42)
    grav = G.BruteForce(eps, G.PREC_FP64_EXACT, ctx)
    p.clear_accelerations()
    grav.compute_accelerations(p)
    q.clear_accelerations()
    O.bf_serial(q, eps)
    kdk = G.LeapfrogKDK()
    g = O.gravity(O.GRAV_BF, eps)
    for _ in range(50):
        kdk.step(p, grav, dt)
        O.kdk_step(q, g, dt)
    for a, b in (("x", "x"), ("vx", "vx"), ("z", "z"), ("ax", "ax")):
        assert np.array_equal(getattr(p, a), getattr(q, b)), a


def test_resident_steps_match_plummer_artifact(ctx, golden):
    """The reference's m1_plummer_1k_diag.csv, reproduced by the GPU path: N=1000,
    seed 42, suggested eps/dt, 1000 device-resident KDK steps, diagnostics every 100."""
    sc = G.PlummerSphere(1000, seed=42)
    eps, dt = sc.suggested_softening(), sc.suggested_dt()
    p = sc.generate()
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_FP64_EXACT, eps)
    rows = golden["m1_plummer_1k_diag.csv"]["rows"]
    d0 = ctx.diagnostics(eps)
    assert abs(d0.total_energy - rows[0][4]) <= 1e-10 * abs(rows[0][4])
    for k in range(1, 11):
        ctx.kdk_steps(G.ALGO_DIRECT, G.PREC_FP64_EXACT, eps, 0.0, dt, 100)
        d = ctx.diagnostics(eps)
        for got, want in ((d.kinetic_energy, rows[k][2]), (d.potential_energy, rows[k][3]),
                          (d.total_energy, rows[k][4])):
            assert abs(got - want) <= 1e-10 * abs(want), (k, got, want)


def test_kepler_artifact_first_rows(ctx, golden):
    """m1_kepler_diag.csv rows 1-2 (2e4 steps of the e=0.5 orbit) on the GPU."""
    tb = G.TwoBody(0.5, 0.5, 1.0)
    p = tb.generate()
    eps, dt = tb.suggested_softening(), tb.suggested_dt()
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_FP64_EXACT, eps)
    rows = golden["m1_kepler_diag.csv"]["rows"]
    for k in (1, 2):
        ctx.kdk_steps(G.ALGO_DIRECT, G.PREC_FP64_EXACT, eps, 0.0, dt, 10000)
        d = ctx.diagnostics(eps)
        assert abs(d.kinetic_energy - rows[k][2]) <= 1e-10 * abs(rows[k][2])
        assert abs(d.total_energy - rows[k][4]) <= 1e-10 * abs(rows[k][4])


def test_diagnostics_vs_oracle(ctx):
    n = 3000
    p = G.PlummerSphere(n, seed=8).generate()
    q = O.plummer(n, 8)
    eps = 0.03
    ctx.set_state(p)
    d = ctx.diagnostics(eps)
    e = O.diagnostics(q, eps)
    assert abs(d.kinetic_energy - e["kinetic_energy"]) <= 1e-12 * abs(e["kinetic_energy"])
    assert abs(d.potential_energy - e["potential_energy"]) <= 1e-12 * abs(e["potential_energy"])
    assert np.allclose(d.angular_momentum, e["angular_momentum"], rtol=1e-12, atol=1e-15)
    assert abs(d.virial_ratio - e["virial_ratio"]) < 1e-12


def test_mixed_resident_energy_drift(ctx):
    """Mixed precision KDK over 1000 steps keeps |dE/E| at the f64 level of the same run."""
    n, eps, dt = 4096, 0.01, 1e-3
    p = G.PlummerSphere(n, seed=1).generate()
    out = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        e0 = ctx.diagnostics(eps).total_energy
        ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 1000)
        out[prec] = abs(ctx.diagnostics(eps).total_energy - e0) / abs(e0)
    print("dE/E fp64 %.3e mixed %.3e" % (out[G.PREC_FP64], out[G.PREC_MIXED]))
    assert out[G.PREC_MIXED] < max(10 * out[G.PREC_FP64], 1e-6)


def test_subset_probe(ctx):
    n = 5000
    p = G.PlummerSphere(n, seed=2).generate()
    ctx.set_state(p)
    idx = np.array([0, 17, 4999, 2500])
    sub = ctx.direct_subset(idx, 0.02)
    full = oracle_acc(O.plummer(n, 2), 0.02)
    assert np.array_equal(sub, full[idx])


def test_fault_injection(ctx):
    """Host-side injected faults come back as status codes; the context stays usable."""
    p = G.PlummerSphere(100, seed=1).generate()
    ctx.set_state(p)
    ctx.set_fault("launch")
    with pytest.raises(G.GvsError) as ei:
        ctx.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, 0.01)
    assert ei.value.status == 6
    ctx.set_fault("nan@3")
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, 0.01)
    with pytest.raises(G.GvsError) as ei:
        ctx.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, 0.01, 0.0, 1e-3, 10)
    assert ei.value.status == 6
    ctx.set_fault("none")
    ctx.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, 0.01, 0.0, 1e-3, 2)
    ctx.sync()
    with pytest.raises(G.GvsError):
        ctx.set_fault("bogus")


SHAPES = [(256, 4, 2, 2), (128, 4, 4, 4), (128, 4, 4, 2), (128, 4, 4, 8), (128, 4, 4, 16), (256, 4, 2, 4),
          (256, 4, 2, 8), (256, 4, 2, 16), (512, 4, 1, 8), (512, 4, 1, 2)]


def test_every_shape_within_mixed_bar(ctx):
    """Each compiled pair-kernel shape meets the mixed bar against the exact f64 sum,
    and shapes that differ only in the loop unroll give identical forces.  n is
    large enough (>= 64 tiles of 512) that no shape falls back to 128 tiles."""
    n, eps = 40000, 0.005
    p = G.PlummerSphere(n=n, seed=11).generate()
    exact = gpu_acc(ctx, p, eps, G.PREC_FP64_EXACT)
    by_tile = {}
    try:
        for sh in SHAPES:
            ctx.set_direct_shape(*sh)
            a = gpu_acc(ctx, p, eps, G.PREC_MIXED)
            assert rel_rms(a, exact) <= 1e-6, sh
            if sh[0] in by_tile:
                assert np.array_equal(a, by_tile[sh[0]]), sh
            else:
                by_tile[sh[0]] = a
        with pytest.raises(G.GvsError):
            ctx.set_direct_shape(96, 4, 2, 8)
    finally:
        ctx.set_direct_shape(*SHAPES[0])


def test_large_tiles_fall_back_on_small_systems(ctx):
    """Below 64 tiles a larger shape runs with 128-particle tiles: same forces."""
    p = G.PlummerSphere(n=3000, seed=12).generate()
    try:
        ctx.set_direct_shape(128, 4, 4, 8)
        a128 = gpu_acc(ctx, p, 0.01, G.PREC_MIXED)
        ctx.set_direct_shape(256, 4, 2, 8)  # falls back to (128, 4, 4, 8)
        a256 = gpu_acc(ctx, p, 0.01, G.PREC_MIXED)
        assert np.array_equal(a128, a256)
    finally:
        ctx.set_direct_shape(*SHAPES[0])



@pytest.mark.parametrize("prec", [G.PREC_FP64_EXACT, G.PREC_MIXED])
def test_graph_replayed_steps_equal_eager_steps(ctx, prec):
    """gvs_kdk_steps replays one captured direct-sum step as a CUDA graph; the
    trajectory is bit-identical to stepping one call at a time (eager)."""
    p = G.PlummerSphere(3000, seed=21).generate()
    eps, dt = 0.01, 1e-3
    runs = []
    for graph in (False, True):
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
        if graph:
            ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 12)
        else:
            for _ in range(12):
                ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 1)
        q = G.Particles(p.count)
        ctx.get_state(q)
        runs.append(q)
    for f in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
        assert np.array_equal(getattr(runs[0], f), getattr(runs[1], f)), f
    # a second call reuses the graph; a new dt recaptures it
    ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, 3)
    ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, 0.5 * dt, 3)
    ctx.sync()


def test_mixed_at_full_size(ctx):
    """N = 2^20 (the headline workload): mixed forces on 2048 random targets within
    1e-6 relative RMS of the exact f64 sum, and the size-independent momentum
    check: sum m a = 0 up to the f32 rounding of the pair terms."""
    n = 1 << 20
    p = G.PlummerSphere(n, seed=1).generate()
    eps = 0.04 / n ** (1.0 / 3.0)
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
    q = G.Particles(n)
    ctx.get_state(q)
    idx = np.sort(np.random.default_rng(4).choice(n, 2048, replace=False))
    ref = ctx.direct_subset(idx, eps)
    err = rel_rms(q.acc()[idx], ref)
    print(f"N=2^20 mixed vs exact on 2048 targets: rel RMS {err:.2e}")
    assert err <= 1e-6
    ma = (q.acc() * q.mass[:, None]).sum(0)
    scale = (np.abs(q.acc()) * q.mass[:, None]).sum(0)
    assert np.all(np.abs(ma) <= 1e-6 * scale), (ma, scale)


def test_bounded_wait_reports_timeout_and_context_survives(ctx):
    """A device wait that runs out returns GVS_ERR_TIMEOUT through the error word
    (no trap, no hang), and the same context computes forces right after."""
    from gravis_gb300 import _lib as L
    st = ctx._lib.gvs_check_bounded_wait(ctx.h, 1000)
    assert st == L.ERR_TIMEOUT
    assert ctx._lib.gvs_check_bounded_wait(ctx.h, 0) == L.ERR_INVALID_ARG
    p = G.PlummerSphere(500, seed=2).generate()
    a = gpu_acc(ctx, p, 0.01, G.PREC_FP64_EXACT)
    q = O.plummer(500, 2)
    q.clear_accelerations()
    O.bf_gather(q, 0.01)
    assert np.array_equal(a, q.acc())


"""PlummerSphere::generate on the GPU (gvs_ic_plummer_device,
crates/sim-core/src/scenarios/plummer_sphere.rs:13-133) against the host generator
(gvs_ic_plummer, whose arrays equal the oracle's and reproduce the reference's m1 Plummer
CSV): the same ChaCha20 stream and draw sequence -- a particle that started one word off
would differ completely -- and values within a few ulps (CUDA's pow/sin/cos against the C
library's; the COM shift sums in another order).
"""
import time

import numpy as np
import pytest

import gravis_gb300 as G

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz")


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("n,seed,a,mass", [(1, 1, 1.0, 1.0), (2, 7, 1.0, 1.0), (1000, 42, 1.0, 1.0),
                                           (20000, 3, 2.5, 7.0), (1 << 20, 1, 1.0, 1.0)])
def test_device_plummer_matches_host(ctx, n, seed, a, mass):
    t0 = time.perf_counter()
    host = G.PlummerSphere(n, scale_radius=a, total_mass=mass, seed=seed).generate()
    t1 = time.perf_counter()
    ctx.ic_plummer_device(n, seed, a, mass)
    ctx.sync()
    t2 = time.perf_counter()
    q = G.Particles(n)
    ctx.get_state(q)
    worst = 0.0
    for f in FIELDS:
        h, d = getattr(host, f), getattr(q, f)
        scale = max(np.abs(h).max(), 1e-300)
        err = float(np.abs(d - h).max()) / scale
        worst = max(worst, err)
        assert err <= 1e-13, (f, err)
    print(f"n={n} seed={seed}: max |device - host| / max |host| = {worst:.1e}; "
          f"host {1e3 * (t1 - t0):.1f} ms, device {1e3 * (t2 - t1):.1f} ms")


@pytest.mark.parametrize("n,seed", [(2, 7), (1001, 7), (1 << 20, 7)])
def test_device_collision_matches_host(ctx, n, seed):
    """The Barnes-Hut workload's ICs (two Plummer spheres from one stream, gvs_ic_collision)."""
    host = G.collision(n, seed=seed)
    ctx.ic_collision_device(n, seed)
    q = G.Particles(n)
    ctx.get_state(q)
    for f in FIELDS:
        h, d = getattr(host, f), getattr(q, f)
        err = float(np.abs(d - h).max()) / max(np.abs(h).max(), 1e-300)
        assert err <= 1e-13, (f, err)


def test_device_plummer_resident_state_steps(ctx):
    """The generated state (masses total_mass / n included) is a normal resident state:
    the direct-sum KDK runs on it and gives the trajectory of the host ICs uploaded."""
    n, seed = 4096, 9
    eps, dt = 0.01, 1e-3
    host = G.PlummerSphere(n, seed=seed).generate()
    c2 = G.Context(0)
    try:
        c2.set_state(host)
        c2.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
        c2.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 10)
        ref = G.Particles(n)
        c2.get_state(ref)
    finally:
        c2.close()
    ctx.ic_plummer_device(n, seed)
    ctx.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, eps)
    ctx.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, eps, 0.0, dt, 10)
    q = G.Particles(n)
    ctx.get_state(q)
    assert np.abs(q.x - ref.x).max() <= 1e-10 * np.abs(ref.x).max()


def test_device_plummer_rejects_bad_arguments(ctx):
    with pytest.raises(G.GvsError):
        ctx.ic_plummer_device(0, 1)
    with pytest.raises(G.GvsError):
        ctx.ic_plummer_device(10, 1, scale_radius=-1.0)
    with pytest.raises(G.GvsError):
        ctx.ic_collision_device(1, 7)

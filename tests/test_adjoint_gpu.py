"""Adjoint (reverse-mode) gradients through the GPU KDK integrator.

No reference counterpart: the forward map is LeapfrogKDK::step
(crates/sim-core/src/integrator.rs:42-76) with BruteForce forces.  Checked
against central finite differences of the f64 forward run (step 1e-6) along
random directions, for dL/dx0, dL/dv0 and dL/dm, with
L = sum_i m_i |x_i(T) - x*_i|^2.  Bars: f64 adjoint vs f64 FD <= 1e-6
relative; mixed-precision adjoint vs f64 adjoint <= 1e-4 relative.
"""
import numpy as np
import pytest

import gravis_gb300 as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def forward_loss(ctx, p, xstar, eps, dt, nsteps, prec=G.PREC_FP64):
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_DIRECT, prec, eps)
    ctx.kdk_steps(G.ALGO_DIRECT, prec, eps, 0.0, dt, nsteps)
    q = G.Particles(p.count)
    ctx.get_state(q)
    x = np.stack([q.x, q.y, q.z], 1)
    return float((p.mass[:, None] * (x - xstar) ** 2).sum()), x


def adjoint_grad(ctx, p, xstar, eps, dt, nsteps, prec, every):
    ctx.set_state(p)
    ctx.adjoint_forward(prec, eps, dt, nsteps, every)
    q = G.Particles(p.count)
    ctx.get_state(q)
    x = np.stack([q.x, q.y, q.z], 1)
    dl_dx = 2.0 * p.mass[:, None] * (x - xstar)
    g = ctx.adjoint_backward(dl_dx)
    g["m"] = g["m"] + ((x - xstar) ** 2).sum(1)  # the loss's own mass dependence
    return g


def setup(n, seed, eps, dt, nsteps, ctx):
    p = G.PlummerSphere(n, seed=seed).generate()
    _, xT = forward_loss(ctx, p, np.zeros((n, 3)), eps, dt, nsteps)
    xstar = xT + 0.01 * np.random.default_rng(seed).standard_normal((n, 3))
    return p, xstar


def perturbed(p, which, u, d):
    q = p.copy()
    if which == "x":
        q.x += d * u[:, 0]; q.y += d * u[:, 1]; q.z += d * u[:, 2]
    elif which == "v":
        q.vx += d * u[:, 0]; q.vy += d * u[:, 1]; q.vz += d * u[:, 2]
    else:
        q.mass += d * u
    return q


def test_fp64_adjoint_vs_finite_differences(ctx):
    n, eps, dt, nsteps = 256, 0.05, 1e-3, 60
    p, xstar = setup(n, 11, eps, dt, nsteps, ctx)
    g = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_FP64, every=20)
    rng = np.random.default_rng(3)
    delta = 1e-6
    for which in ("x", "v", "m"):
        for _ in range(3):
            u = rng.standard_normal((n, 3)) if which != "m" else rng.standard_normal(n) * p.mass
            lp, _ = forward_loss(ctx, perturbed(p, which, u, delta), xstar, eps, dt, nsteps)
            lm, _ = forward_loss(ctx, perturbed(p, which, u, -delta), xstar, eps, dt, nsteps)
            fd = (lp - lm) / (2 * delta)
            ad = float((g[which] * u).sum())
            print(f"{which}: adjoint {ad:.12e} fd {fd:.12e} rel {abs(ad - fd) / abs(fd):.2e}")
            assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-12


def test_mixed_adjoint_vs_fp64_adjoint(ctx):
    n, eps, dt, nsteps = 4096, 0.01, 1e-3, 200
    p, xstar = setup(n, 5, eps, dt, nsteps, ctx)
    g64 = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_FP64, every=50)
    gmx = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_MIXED, every=50)
    for which in ("x", "v", "m"):
        rel = np.linalg.norm(gmx[which] - g64[which]) / np.linalg.norm(g64[which])
        print(f"mixed vs f64 adjoint {which}: {rel:.2e}")
        assert rel <= 1e-4


def test_checkpoint_interval_independent(ctx):
    n, eps, dt, nsteps = 512, 0.02, 1e-3, 100
    p, xstar = setup(n, 2, eps, dt, nsteps, ctx)
    a = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_FP64, every=1)
    b = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_FP64, every=100)
    for which in ("x", "v", "m"):
        assert np.linalg.norm(a[which] - b[which]) <= 1e-9 * np.linalg.norm(a[which])


def test_backward_restores_initial_state(ctx):
    n, eps, dt, nsteps = 300, 0.02, 1e-3, 30
    p, xstar = setup(n, 4, eps, dt, nsteps, ctx)
    adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_MIXED, every=10)
    q = G.Particles(n)
    ctx.get_state(q)
    assert np.array_equal(q.x, p.x) and np.array_equal(q.vz, p.vz)


def test_fp64_adjoint_vs_finite_differences_4096(ctx):
    """N = 4096 Plummer, eps 0.01, dt 1e-3, 200 steps, f64 checkpoints every 100:
    the f64 adjoint's directional derivative along 8 random directions of
    (x0, v0, m) against f64 central differences with step 1e-6, within 1e-5."""
    n, eps, dt, nsteps = 4096, 0.01, 1e-3, 200
    p, xstar = setup(n, 42, eps, dt, nsteps, ctx)
    g = adjoint_grad(ctx, p, xstar, eps, dt, nsteps, G.PREC_FP64, every=100)
    rng = np.random.default_rng(7)
    delta = 1e-6
    errs = []
    for _ in range(8):
        ux, uv, um = rng.standard_normal((n, 3)), rng.standard_normal((n, 3)), rng.standard_normal(n) * p.mass
        plus = perturbed(perturbed(perturbed(p, "x", ux, delta), "v", uv, delta), "m", um, delta)
        minus = perturbed(perturbed(perturbed(p, "x", ux, -delta), "v", uv, -delta), "m", um, -delta)
        lp, _ = forward_loss(ctx, plus, xstar, eps, dt, nsteps)
        lm, _ = forward_loss(ctx, minus, xstar, eps, dt, nsteps)
        fd = (lp - lm) / (2 * delta)
        ad = float((g["x"] * ux).sum() + (g["v"] * uv).sum() + (g["m"] * um).sum())
        errs.append(abs(ad - fd) / abs(fd))
    print(f"8 directions: relative error max {max(errs):.2e}, median {np.median(errs):.2e}")
    assert max(errs) <= 1e-5, errs


@pytest.mark.parametrize("prec", [G.PREC_FP64, G.PREC_MIXED])
def test_checkpoints_as_snapshots_restart_backward(ctx, prec, tmp_path):
    """The forward run's checkpoints, written as NBODY003 snapshots (snapshot.rs:40-65)
    and read into a fresh context, give the same gradients bit for bit; each checkpoint
    is the state of a plain KDK run of that many steps."""
    n, eps, dt, nsteps, every = 384, 0.05, 1e-3, 250, 100
    p, xstar = setup(n, 5, eps, dt, nsteps, ctx)
    ctx.set_state(p)
    ctx.adjoint_forward(prec, eps, dt, nsteps, every)
    assert ctx.adjoint_checkpoint_steps() == [0, 100, 200, 250]
    paths = ctx.adjoint_save_checkpoints(str(tmp_path), p)
    q = G.Particles(n)
    ctx.get_state(q)
    x = np.stack([q.x, q.y, q.z], 1)
    dl_dx = 2.0 * p.mass[:, None] * (x - xstar)
    dl_dv = 0.1 * np.random.default_rng(2).standard_normal((n, 3))
    g1 = ctx.adjoint_backward(dl_dx, dl_dv)
    # a snapshot read back holds the checkpoint (time = step * dt, the run's eps and dt)
    with open(paths[1], "rb") as fh:
        s = G.Snapshot.read_from(fh)
    assert (s.step, s.time, s.softening, s.dt) == (100, 100 * dt, eps, dt)
    xs, vs = ctx.adjoint_checkpoint(1)
    assert np.array_equal(np.stack([s.particles.x, s.particles.y, s.particles.z], 1), xs)
    assert np.array_equal(np.stack([s.particles.vx, s.particles.vy, s.particles.vz], 1), vs)
    assert np.array_equal(s.particles.mass, p.mass)
    # checkpoint 1 is the state after 100 plain KDK steps
    _, x100 = forward_loss(ctx, p, xstar, eps, dt, 100, prec)
    assert np.array_equal(x100, xs)
    c2 = G.Context(0)
    try:
        c2.adjoint_load_checkpoints(reversed(paths), prec)
        g2 = c2.adjoint_backward(dl_dx, dl_dv)
        r = G.Particles(n)
        c2.get_state(r)  # the initial state again, as after the original run's sweep
        assert np.array_equal(r.x, p.x) and np.array_equal(r.vz, p.vz)
        # a set with a gap (0, 100, 250: step 200 missing) is refused
        with pytest.raises(ValueError):
            c2.adjoint_load_checkpoints([paths[0], paths[1], paths[3]], prec)
    finally:
        c2.close()
    for k in ("x", "v", "m"):
        assert np.array_equal(g1[k], g2[k]), k

"""Batched ensembles: many independent systems in one persistent launch.

Each system of the ensemble must evolve exactly as it does on its own through
the single-system mixed-precision path with the same 128-particle tiles (same
Hilbert order, same tiles; only the grouping of source chunks in the f64 reduce
differs), so the bar is 1e-10 relative; against the exact f64 direct sum the
mixed bar 1e-6 holds.
"""
import numpy as np
import pytest

import gravis_gb300 as G
from gravis_gb300.engine import plummer_ensemble

pytestmark = pytest.mark.gpu

EPS = 0.01


@pytest.fixture(scope="module")
def ctx():
    c = G.Context(0)
    yield c
    c.close()


def split(p, sizes):
    out, o = [], 0
    for n in sizes:
        q = G.Particles(int(n))
        for f in ("x", "y", "z", "vx", "vy", "vz", "mass", "ax", "ay", "az"):
            getattr(q, f)[:] = getattr(p, f)[o:o + n]
        out.append(q)
        o += n
    return out


def single_context():
    c = G.Context(0)
    c.set_direct_shape(128, 4, 4, 4)  # the ensemble's tile size
    return c


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def ens():
    sizes = G.ensemble_sizes(24, seed=7, lo=100, hi=3000)
    return sizes, plummer_ensemble(sizes)


def test_ensemble_forces_match_single_systems(ctx, ens):
    sizes, p = ens
    ctx.set_state(p)
    ctx.ensemble_setup(sizes, EPS)
    ctx.ensemble_forces()
    q = G.Particles(p.count)
    ctx.get_state(q)
    single = single_context()
    try:
        for k, s in enumerate(split(q, sizes)):
            r = split(p, sizes)[k]
            single.set_state(r)
            single.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, EPS)
            a = G.Particles(r.count)
            single.get_state(a)
            assert rel(s.acc(), a.acc()) <= 1e-10, k
            single.compute_forces(G.ALGO_DIRECT, G.PREC_FP64_EXACT, EPS)
            single.get_state(a)
            assert rel(s.acc(), a.acc()) <= 1e-6, k
    finally:
        single.close()


def test_graph_equals_eager_and_single_runs(ctx, ens):
    sizes, p = ens
    dt, steps = 1e-3, 20
    runs = []
    for use_graph in (False, True):
        ctx.set_state(p)
        ctx.ensemble_setup(sizes, EPS)
        ctx.ensemble_forces()
        ctx.ensemble_kdk_steps(dt, steps, use_graph)
        q = G.Particles(p.count)
        ctx.get_state(q)
        runs.append(q)
    assert np.array_equal(runs[0].x, runs[1].x) and np.array_equal(runs[0].vz, runs[1].vz)
    single = single_context()
    try:
        for k, (s, r) in enumerate(zip(split(runs[1], sizes), split(p, sizes))):
            single.set_state(r)
            single.compute_forces(G.ALGO_DIRECT, G.PREC_MIXED, EPS)
            single.kdk_steps(G.ALGO_DIRECT, G.PREC_MIXED, EPS, 0.0, dt, steps)
            a = G.Particles(r.count)
            single.get_state(a)
            assert rel(np.stack([s.x, s.y, s.z]), np.stack([a.x, a.y, a.z])) <= 1e-10, k
    finally:
        single.close()


def test_ensemble_rejects_bad_sizes(ctx, ens):
    sizes, p = ens
    ctx.set_state(p)
    with pytest.raises(G.GvsError):
        ctx.ensemble_setup(np.array(sizes[:-1]), EPS)
    with pytest.raises(G.GvsError):
        ctx.ensemble_setup(np.concatenate([sizes[:-1], [0]]), EPS)

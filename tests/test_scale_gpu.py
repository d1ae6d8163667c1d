"""Parity at the benchmark sizes: the GPU tree, the Barnes-Hut walk that makes
the reference's opening decisions, and the SPH pipeline, against the oracle's
restatement of sim-core on the workloads' own initial conditions.

- Octree (Octree::rebuild, crates/sim-core/src/octree.rs:156-239) of two
  Plummer spheres (seed 7) at N = 2^22 and 2^24: node count, depth-first leaf
  order (= the GPU sort order) and every particle's octant path, bit-exact.
  This runs the certified integer key path where it matters (about 95 % of
  the particles skip the f64 replay).
- Mixed BH walk (barnes_hut.rs:44-135) at N = 2^22, theta 0.5 and 0.7,
  eps 1e-3: 4096 random targets against the oracle's BarnesHut on the same
  tree, within 1e-6 relative RMS; and exactly as many terms as the f64 walk
  (the same opening decisions for all 2^22 particles).
- SPH (neighbors.rs:56-119, density.rs:42-157, forces.rs:80-225) on the
  rho ~ 1/r gas sphere at N = 2^18 and 2^20: neighbour lists identical in set
  and order; f64 density, h, Omega, P, c within 1e-12 and a, du/dt, div v,
  max mu, d alpha/dt within 1e-10; the mixed form within 1e-6.
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


def to_oracle(p):
    q = O.Particles(p.count)
    pairs = (("x", "x"), ("y", "y"), ("z", "z"), ("vx", "vx"), ("vy", "vy"), ("vz", "vz"), ("ax", "ax"), ("ay", "ay"),
             ("az", "az"), ("mass", "mass"), ("density", "density"), ("pressure", "pressure"),
             ("internal_energy", "u"), ("du_dt", "du_dt"), ("smoothing_length", "h"), ("sound_speed", "cs"),
             ("alpha_visc", "alpha"), ("particle_type", "ptype"))
    for a, b in pairs:
        getattr(q, b)[:] = getattr(p, a)
    return q


def path_masks(depth):
    """Masks of the octant-path bits above each leaf's depth (3 bits per level,
    levels 1..21 in the high word, 22..42 in the low word, left-aligned)."""
    depth = np.asarray(depth, dtype=np.int64)
    one = np.uint64(1)
    kh = np.minimum(depth, 21).astype(np.uint64)
    kl = np.clip(depth - 21, 0, 21).astype(np.uint64)
    mhi = ((one << (np.uint64(3) * kh)) - one) << (np.uint64(63) - np.uint64(3) * kh)
    mlo = ((one << (np.uint64(3) * kl)) - one) << (np.uint64(63) - np.uint64(3) * kl)
    return mhi, mlo


@pytest.mark.parametrize("n", [1 << 22, 1 << 24])
def test_tree_bit_exact_at_benchmark_size(ctx, n):
    p = G.collision(n, seed=7)
    ctx.set_state(p)
    t = ctx.tree_export()
    ref = O.octree_leaves(to_oracle(p))
    assert t["nnodes"] == ref["nnodes"]
    leaves = t["count"] > 0
    assert int(leaves.sum()) == ref["nleaves"] == n
    first = t["first"][leaves]
    # depth-first leaf order == the GPU's sorted order
    assert np.array_equal(t["order"][first], ref["order"])
    assert np.array_equal(t["level"][leaves].astype(np.int32), ref["depth"])
    mhi, mlo = path_masks(ref["depth"])
    assert np.array_equal(t["keys"][0][first] & mhi, ref["path_hi"])
    assert np.array_equal(t["keys"][1][first] & mlo, ref["path_lo"])
    print(f"N={n}: {ref['nnodes']} nodes, deepest leaf {int(ref['depth'].max())}, "
          f"{int((ref['depth'] > 21).sum())} leaves below depth 21")


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_bh_parity_walk_at_benchmark_size(ctx, theta):
    n, eps = 1 << 22, 1e-3
    p = G.collision(n, seed=7)
    idx = np.sort(np.random.default_rng(11).choice(n, 4096, replace=False))
    ref = O.bh_subset(to_oracle(p), eps, theta, idx)
    q = p.copy()
    q.clear_accelerations()
    G.BarnesHut(eps, theta, G.PREC_MIXED, ctx).compute_accelerations(q)
    got = q.acc()[idx]
    rel = float(np.sqrt(((got - ref) ** 2).sum() / (ref ** 2).sum()))
    per = np.sqrt(((got - ref) ** 2).sum(1) / (ref ** 2).sum(1))
    print(f"theta={theta}: mixed walk vs oracle BarnesHut rel RMS {rel:.2e}, per-particle max {per.max():.2e}")
    assert rel <= 1e-6, rel


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_bh_mixed_walk_terms_equal_f64_walk_at_benchmark_size(ctx, theta):
    """At N = 2^22 the mixed walk sums exactly the f64 walk's terms (the reference's
    decisions, barnes_hut.rs:85-91): the f32 test with its certified band never decides
    a node the other way."""
    n, eps = 1 << 22, 1e-3
    p = G.collision(n, seed=7)
    terms = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        q = p.copy()
        q.clear_accelerations()
        try:
            ctx.profile(True)
            G.BarnesHut(eps, theta, prec, ctx).compute_accelerations(q)
            terms[prec] = ctx.profile_read()["bh_walk_terms"]
        finally:
            ctx.profile(False)
    print(f"theta={theta}: {terms[G.PREC_MIXED]} terms (f64 walk {terms[G.PREC_FP64]})")
    assert terms[G.PREC_MIXED] == terms[G.PREC_FP64] > 0


def csr_positions(start, count):
    """Flat positions of every entry of a CSR list whose rows start anywhere."""
    count = np.asarray(count, dtype=np.int64)
    row_first = np.cumsum(count) - count
    total = int(count.sum())
    return np.repeat(np.asarray(start, dtype=np.int64), count) + (np.arange(total) - np.repeat(row_first, count))


def rel(a, b):
    d = np.sqrt(((a - b) ** 2).sum())
    s = np.sqrt((b ** 2).sum())
    return d / s if s > 0 else d


@pytest.fixture(scope="module", params=[1 << 18, 1 << 20], ids=["n262144", "n1048576"])
def sph_case(request):
    n = request.param
    p = G.gas_sphere_1r(n)
    q = to_oracle(p)
    s = O.Sph()
    s.compute(q)
    return n, p, q, s


def test_sph_f64_at_benchmark_size(ctx, sph_case):
    n, p0, q, s = sph_case
    p = p0.copy()
    sph = G.SphSolver(ctx)
    inter = sph.compute(p)
    start, count, idx = sph.neighbors()
    ostart, oend, oidx = s.neighbor_lists(n)
    assert np.array_equal(count.astype(np.int64), (oend - ostart).astype(np.int64))
    assert np.array_equal(idx[csr_positions(start, count)], oidx[csr_positions(ostart, oend - ostart)])
    for a, b in (("density", "density"), ("smoothing_length", "h"), ("pressure", "pressure"),
                 ("sound_speed", "cs")):
        assert rel(getattr(p, a), getattr(q, b)) <= 1e-12, (a, rel(getattr(p, a), getattr(q, b)))
    assert rel(inter.omega, s.array("omega", n)) <= 1e-12
    for a in ("ax", "ay", "az", "du_dt"):
        assert rel(getattr(p, a), getattr(q, a)) <= 1e-10, (a, rel(getattr(p, a), getattr(q, a)))
    assert rel(inter.div_v, s.array("div_v", n)) <= 1e-10
    assert rel(inter.max_mu, s.array("max_mu", n)) <= 1e-10
    assert rel(inter.dalpha_dt, s.array("dalpha_dt", n)) <= 1e-10
    print(f"N={n}: {len(idx)} neighbour entries identical; a rel {rel(p.ax, q.ax):.1e}")


def test_sph_mixed_at_benchmark_size(ctx, sph_case):
    n, p0, q, s = sph_case
    p = p0.copy()
    sph = G.SphSolver(ctx)
    sph.params.precision = G.PREC_MIXED
    inter = sph.compute(p)
    start, count, idx = sph.neighbors()
    ostart, oend, oidx = s.neighbor_lists(n)
    assert np.array_equal(idx[csr_positions(start, count)], oidx[csr_positions(ostart, oend - ostart)])
    errs = {a: rel(getattr(p, a), getattr(q, b)) for a, b in
            (("density", "density"), ("smoothing_length", "h"), ("pressure", "pressure"), ("ax", "ax"),
             ("ay", "ay"), ("az", "az"), ("du_dt", "du_dt"))}
    errs["omega"] = rel(inter.omega, s.array("omega", n))
    print(f"N={n} mixed: " + ", ".join(f"{k} {v:.1e}" for k, v in errs.items()))
    for k, v in errs.items():
        assert v <= 1e-6, (k, v)

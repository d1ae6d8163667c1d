"""GPU octree + Barnes-Hut against the oracle's restatement of the reference.

Tree: bit-exact.  The node count, the depth-first leaf order (= the GPU sort
order) and every particle's octant path down to its leaf must equal the
reference tree's (Octree::rebuild, crates/sim-core/src/octree.rs:156-239).
Forces: the f64 walk makes the reference's accept decisions on a bottom-up
centre of mass (a few ulps from the reference's incremental one) and sums
children 0..7 instead of 7..0, so it agrees with the oracle's BarnesHut to
<= 1e-12 relative RMS; the f32 walk within 1e-4 of the f64 walk; the mixed walk
(f32 terms on float-float separations, the reference's opening decisions)
within 1e-6 of the oracle's BarnesHut and of the f64 walk.
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


def to_oracle(p):
    q = O.Particles(p.count)
    for a, b in (("x", "x"), ("y", "y"), ("z", "z"), ("vx", "vx"), ("vy", "vy"), ("vz", "vz"), ("mass", "mass")):
        getattr(q, b)[:] = getattr(p, a)
    return q


def lattice(n_side, spacing):
    p = G.Particles(n_side ** 3)
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                p.x[k], p.y[k], p.z[k], p.mass[k] = ix * spacing, iy * spacing, iz * spacing, 1.0
                k += 1
    return p


def close_pairs(n=2000, k=40, sep=1e-9):
    """n Plummer particles plus k copies of the first k moved by sep*(1..k) in x: pairs
    that share all 21 high key levels and split between depths 22 and 42."""
    p = G.PlummerSphere(n, seed=4).generate()
    q = G.Particles(n + k)
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        getattr(q, f)[:n] = getattr(p, f)
        getattr(q, f)[n:] = getattr(p, f)[:k]
    q.x[n:] += sep * np.arange(1, k + 1)
    return q


def cases():
    return {
        "close_pairs": close_pairs(),
        "plummer1000": G.PlummerSphere(1000, seed=42).generate(),
        "plummer20000": G.PlummerSphere(20000, seed=3).generate(),
        "collision4096": G.collision(4096, seed=7),
        "lattice8": lattice(8, 0.5),  # exact octant-boundary ties
        "two": G.TwoBody(0.5, 0.5, 1.0).generate(),
        "one": G.PlummerSphere(1, seed=1).generate(),
    }


@pytest.mark.parametrize("name", list(cases().keys()))
def test_tree_matches_reference(ctx, name):
    p = cases()[name]
    ctx.set_state(p)
    t = ctx.tree_export()
    ref = O.octree_leaves(to_oracle(p))
    assert t["nnodes"] == ref["nnodes"]
    leaves = t["count"] > 0
    assert int(leaves.sum()) == ref["nleaves"] == p.count
    # depth-first leaf order == sorted order of the GPU
    assert np.array_equal(t["order"][t["first"][leaves]], ref["order"])
    assert np.array_equal(t["level"][leaves].astype(np.int32), ref["depth"])
    # octant paths, bit-exact, truncated at each leaf's depth
    hi, lo = t["keys"][0][t["first"][leaves]], t["keys"][1][t["first"][leaves]]
    def masks(k):
        k = int(k)
        if k <= 21:
            return ((1 << (3 * k)) - 1) << (63 - 3 * k), 0
        return (1 << 63) - 1, ((1 << (3 * (k - 21))) - 1) << (63 - 3 * (k - 21))
    mk = [masks(k) for k in ref["depth"]]
    mask_hi = np.array([a for a, _ in mk], dtype=np.uint64)
    mask_lo = np.array([b for _, b in mk], dtype=np.uint64)
    assert np.array_equal(hi & mask_hi, ref["path_hi"])
    assert np.array_equal(lo & mask_lo, ref["path_lo"])
    # moments: the root holds the total mass and centre of mass
    m = p.mass
    assert abs(t["mass"][0] - m.sum()) <= 1e-12 * m.sum()
    com = np.array([(m * p.x).sum(), (m * p.y).sum(), (m * p.z).sum()]) / m.sum()
    assert np.allclose(t["com"][:, 0], com, rtol=0, atol=1e-12 * max(1.0, np.abs(p.x).max()))


@pytest.mark.parametrize("theta", [0.0, 0.3, 0.5, 0.7, 1.0])
@pytest.mark.parametrize("name", ["plummer1000", "collision4096", "lattice8"])
def test_bh_f64_vs_oracle(ctx, name, theta):
    p = cases()[name]
    eps = 0.05
    q = p.copy()
    q.clear_accelerations()
    G.BarnesHut(eps, theta, G.PREC_FP64, ctx).compute_accelerations(q)
    r = to_oracle(p)
    O.bh(r, eps, theta)
    assert rel_rms(q.acc(), r.acc()) <= 1e-12, rel_rms(q.acc(), r.acc())


def test_bh_theta_zero_is_bf(ctx):
    """barnes_hut.rs:219-265 on the GPU: theta = 0 equals BruteForce within 1e-12."""
    pts = [(0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 2.0), (0.0, 1.0, 0.0, 1.5), (-1.0, -1.0, 0.5, 0.5),
           (0.5, 0.5, -0.5, 3.0)]
    p = G.Particles(5)
    for i, (x, y, z, m) in enumerate(pts):
        p.x[i], p.y[i], p.z[i], p.mass[i] = x, y, z, m
    a = p.copy()
    G.BarnesHut(0.05, 0.0, G.PREC_FP64, ctx).compute_accelerations(a)
    b = p.copy()
    G.BruteForce(0.05, G.PREC_FP64_EXACT, ctx).compute_accelerations(b)
    assert np.max(np.abs(a.acc() - b.acc())) < 1e-12


def test_bh_accuracy_table(ctx, golden):
    """m3_accuracy.csv from the GPU walk: BH vs BF relative error at N=1000, seed 42, eps 0.05."""
    p = G.PlummerSphere(1000, seed=42).generate()
    bf = p.copy()
    G.BruteForce(0.05, G.PREC_FP64_EXACT, ctx).compute_accelerations(bf)
    a = bf.acc()
    for row in golden["m3_accuracy.csv"]["rows"]:
        q = p.copy()
        G.BarnesHut(0.05, row[0], G.PREC_FP64, ctx).compute_accelerations(q)
        m2 = (a * a).sum(1)
        rel = ((q.acc() - a) ** 2).sum(1) / m2
        rms, mx = np.sqrt(rel.sum() / 1000), np.sqrt(rel.max())
        assert f"{rms:.5e}" == f"{row[2]:.5e}", (row[0], rms, row[2])
        assert f"{mx:.5e}" == f"{row[3]:.5e}", (row[0], mx, row[3])


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_bh_f32_walk(ctx, theta):
    """The per-particle f32 walk (the reference's test on f32 positions)."""
    p = G.collision(1 << 16, seed=7)
    eps = 1e-3
    a64 = p.copy()
    G.BarnesHut(eps, theta, G.PREC_FP64, ctx).compute_accelerations(a64)
    a32 = p.copy()
    ctx.set_bh_walk(0)
    try:
        G.BarnesHut(eps, theta, G.PREC_FP32, ctx).compute_accelerations(a32)
    finally:
        ctx.set_bh_walk(-1)
    err = rel_rms(a32.acc(), a64.acc())
    print(f"theta={theta} f32 walk vs f64 walk rel RMS {err:.2e}")
    # f32 absolute positions at |x| ~ 10 resolve separations to ~1e-6; the bound
    # sits two orders of magnitude below the BH approximation error (~5e-3).
    assert err <= 1e-4


@pytest.mark.parametrize("theta", [0.3, 0.5, 0.7])
@pytest.mark.parametrize("name", ["plummer1000", "collision4096", "lattice8"])
def test_bh_mixed_vs_oracle(ctx, name, theta):
    """Mixed walk: same accepted nodes as the reference (f64 rechecks near the
    opening boundary), f32 terms on float-float separations: within 1e-6."""
    p = cases()[name]
    eps = 0.05
    q = p.copy()
    q.clear_accelerations()
    G.BarnesHut(eps, theta, G.PREC_MIXED, ctx).compute_accelerations(q)
    r = to_oracle(p)
    O.bh(r, eps, theta)
    err = rel_rms(q.acc(), r.acc())
    print(f"{name} theta={theta} mixed walk vs oracle BH rel RMS {err:.2e}")
    assert err <= 1e-6, err


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_bh_mixed_walk_large(ctx, theta):
    """At 2^16 (two Plummer spheres 20 apart, eps 1e-3) the mixed walk stays within
    1e-6 of the f64 walk, where the plain f32 walk is ~1e-5 away."""
    p = G.collision(1 << 16, seed=7)
    eps = 1e-3
    a64 = p.copy()
    G.BarnesHut(eps, theta, G.PREC_FP64, ctx).compute_accelerations(a64)
    am = p.copy()
    G.BarnesHut(eps, theta, G.PREC_MIXED, ctx).compute_accelerations(am)
    err = rel_rms(am.acc(), a64.acc())
    print(f"theta={theta} mixed walk vs f64 walk rel RMS {err:.2e}")
    assert err <= 1e-6


def walk_terms(ctx, p, eps, theta, prec):
    """Accelerations and the terms summed by a per-particle walk."""
    q = p.copy()
    q.clear_accelerations()
    try:
        ctx.profile(True)
        G.BarnesHut(eps, theta, prec, ctx).compute_accelerations(q)
        terms = ctx.profile_read()["bh_walk_terms"]
    finally:
        ctx.profile(False)
    return q.acc(), terms


def massless(n=5000):
    p = G.PlummerSphere(n, seed=8).generate()
    p.mass[::7] = 0.0  # one particle in seven: leaves and buckets of zero mass
    return with_duplicates(p, 12, at=7)  # a bucket of massless particles


@pytest.mark.parametrize("theta", [0.3, 0.5, 0.7])
@pytest.mark.parametrize("case", ["collision", "buckets", "close_pairs", "massless", "lattice"])
def test_bh_mixed_walk_makes_the_f64_walks_decisions(ctx, case, theta):
    """The mixed walk decides with the f32 distance of the hi words outside a certified
    band around s/theta (from the pair's own coordinate magnitudes) and with the
    reference's f64 test inside it, so it sums exactly the terms of the f64 walk (the
    reference's decisions): the two walks' term counts agree, and the forces within 1e-6."""
    p = {"collision": lambda: G.collision(1 << 17, seed=7),
         "buckets": lambda: with_duplicates(G.PlummerSphere(3000, seed=5).generate(), 99, at=17),
         "close_pairs": lambda: close_pairs(3000, 40),
         "massless": massless,
         "lattice": lambda: lattice(16, 0.25)}[case]()
    eps = 1e-3 if case == "collision" else 0.01
    a64, n64 = walk_terms(ctx, p, eps, theta, G.PREC_FP64)
    am, nm = walk_terms(ctx, p, eps, theta, G.PREC_MIXED)
    err = rel_rms(am, a64)
    print(f"{case} theta={theta}: {nm} terms (f64 walk {n64}), mixed vs f64 rel RMS {err:.1e}")
    assert nm == n64 > 0
    assert err <= 1e-6, err


def test_bh_vs_direct_subset(ctx):
    """Accuracy of the walk against the exact f64 direct sum on a random subset."""
    n = 1 << 17
    p = G.collision(n, seed=7)
    eps = 1e-3
    ctx.set_state(p)
    idx = np.sort(np.random.default_rng(1).choice(n, 2048, replace=False))
    ref = ctx.direct_subset(idx, eps)
    for theta, bound in ((0.5, 0.01), (0.7, 0.03)):
        q = p.copy()
        G.BarnesHut(eps, theta, G.PREC_FP32, ctx).compute_accelerations(q)
        rel = np.sqrt((((q.acc()[idx] - ref) ** 2).sum(1) / (ref ** 2).sum(1)).mean())
        print(f"theta={theta} BH f32 vs direct f64 per-particle RMS {rel:.3e}")
        assert rel < bound


def with_duplicates(p, k, at=0):
    """p plus k particles at exactly the position of particle `at` (a bucket leaf of k + 1)."""
    q = G.Particles(p.count + k)
    for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
        getattr(q, f)[:p.count] = getattr(p, f)
        getattr(q, f)[p.count:] = getattr(p, f)[at]
    return q


@pytest.mark.parametrize("gsize", [32, 64, 128])
@pytest.mark.parametrize("case", ["plummer", "buckets", "bucket10", "close_pairs"])
def test_bh_group_walk_theta_zero_is_direct(ctx, gsize, case):
    """theta = 0 opens every node, so the group walk is the f32 all-pairs sum,
    including the members of bucket leaves: 100 coincident particles (a bucket
    larger than a group, cut into several groups; a run of equal high key words
    too long for the run sort, built on the full-key path), 10 coincident ones
    (sorted by the run sort), and pairs split below depth 21."""
    p = G.PlummerSphere(3000, seed=5).generate()
    if case == "buckets":
        p = with_duplicates(p, 99, at=17)
    elif case == "bucket10":
        p = with_duplicates(p, 9, at=17)
    elif case == "close_pairs":
        p = close_pairs(3000, 40)
    eps = 0.01
    ref = p.copy()
    G.BruteForce(eps, G.PREC_FP64_EXACT, ctx).compute_accelerations(ref)
    try:
        ctx.set_bh_walk(0)
        pp = p.copy()
        G.BarnesHut(eps, 0.0, G.PREC_FP32, ctx).compute_accelerations(pp)
        ctx.set_bh_walk(gsize)
        q = p.copy()
        G.BarnesHut(eps, 0.0, G.PREC_FP32, ctx).compute_accelerations(q)
    finally:
        ctx.set_bh_walk(-1)
    err, err_pp = rel_rms(q.acc(), ref.acc()), rel_rms(pp.acc(), ref.acc())
    print(f"group {gsize} {case}: theta=0 vs f64 direct rel RMS {err:.2e} (per-particle f32 walk {err_pp:.2e})")
    # the same f32 terms on absolute f32 positions as the per-particle walk, summed
    # in another order: the same accuracy
    assert err <= max(5e-6, 1.5 * err_pp)


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_bh_group_walk_refines_per_particle(ctx, theta):
    """The group test accepts only nodes every particle of the group would accept,
    so the group walk is at least as close to the exact f64 direct sum as the
    per-particle walk."""
    n = 1 << 17
    p = G.collision(n, seed=7)
    eps = 1e-3
    ctx.set_state(p)
    idx = np.sort(np.random.default_rng(1).choice(n, 2048, replace=False))
    ref = ctx.direct_subset(idx, eps)
    errs = {}
    try:
        for g in (0, 32, 64, 128):
            ctx.set_bh_walk(g)
            q = p.copy()
            G.BarnesHut(eps, theta, G.PREC_FP32, ctx).compute_accelerations(q)
            errs[g] = float(np.sqrt((((q.acc()[idx] - ref) ** 2).sum(1) / (ref ** 2).sum(1)).mean()))
    finally:
        ctx.set_bh_walk(-1)
    print(f"theta={theta} per-particle RMS vs f64 direct: " + ", ".join(f"{k}: {v:.3e}" for k, v in errs.items()))
    assert errs[32] <= errs[0] and errs[64] <= errs[0] and errs[128] <= errs[0]


@pytest.mark.parametrize("n", [1, 2, 3, 33, 200])
@pytest.mark.parametrize("eps", [0.0, 0.01])
def test_bh_group_walk_tiny(ctx, n, eps):
    """Tiny systems (a root that is a leaf, one partial group) through the FP32 group walk
    at theta = 0: the f32 all-pairs sum; a lone particle feels nothing."""
    p = G.PlummerSphere(n, seed=21).generate()
    ref = p.copy()
    G.BruteForce(eps, G.PREC_FP64_EXACT, ctx).compute_accelerations(ref)
    q = p.copy()
    G.BarnesHut(eps, 0.0, G.PREC_FP32, ctx).compute_accelerations(q)
    assert np.isfinite(q.acc()).all()
    if n == 1:
        assert not q.acc().any()
    else:
        assert rel_rms(q.acc(), ref.acc()) <= 1e-5


def test_bh_group_walk_unsoftened(ctx):
    """eps = 0: a particle's own leaf adds exactly zero (no 0/0), forces stay finite
    and agree with the f64 walk to f32 accuracy at theta = 0."""
    p = G.PlummerSphere(2000, seed=13).generate()
    ref = p.copy()
    G.BruteForce(0.0, G.PREC_FP64_EXACT, ctx).compute_accelerations(ref)
    q = p.copy()
    G.BarnesHut(0.0, 0.0, G.PREC_FP32, ctx).compute_accelerations(q)
    assert np.isfinite(q.acc()).all()
    assert rel_rms(q.acc(), ref.acc()) <= 1e-4


def test_bh_group_walk_fallback_is_per_particle_walk(ctx):
    """With a budget of one iteration every group falls back to the per-particle walk,
    which must reproduce the per-particle kernel bit for bit."""
    p = G.collision(1 << 15, seed=7)
    eps, theta = 1e-3, 0.5
    ctx.set_bh_walk(0)
    try:
        a = p.copy()
        G.BarnesHut(eps, theta, G.PREC_FP32, ctx).compute_accelerations(a)
        ctx.set_bh_walk(64, 1)
        ctx.profile(True)
        b = p.copy()
        G.BarnesHut(eps, theta, G.PREC_FP32, ctx).compute_accelerations(b)
        pr = ctx.profile_read()
        ctx.profile(False)
    finally:
        ctx.set_bh_walk(-1)
    assert pr["bh_groups"] > 0 and pr["bh_group_fallbacks"] == pr["bh_groups"]
    assert np.array_equal(a.acc(), b.acc())


def test_bh_group_walk_rejects_bad_size(ctx):
    with pytest.raises(G.GvsError):
        ctx.set_bh_walk(48)
    with pytest.raises(G.GvsError):
        ctx.set_bh_walk(64, -1)


def test_bh_deterministic_and_resident_steps(ctx):
    p = G.PlummerSphere(5000, seed=9).generate()
    outs = []
    for _ in range(2):
        ctx.set_state(p)
        ctx.compute_forces(G.ALGO_BH, G.PREC_FP32, 0.01, 0.5)
        ctx.kdk_steps(G.ALGO_BH, G.PREC_FP32, 0.01, 0.5, 1e-3, 20)
        q = G.Particles(p.count)
        ctx.get_state(q)
        outs.append(q.x.copy())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("gsize", [64, 128])
def test_bh_group_walk_kdk_energy(ctx, gsize):
    """The FP32 group walk over 500 KDK steps (Plummer N=2000, theta 0.5, dt 1e-3) conserves
    energy at least as well as the reference's f64 walk on the same system."""
    p = G.PlummerSphere(2000, seed=42).generate()
    eps = 0.05
    drift = {}
    try:
        for name, prec, g in (("f64", G.PREC_FP64, -1), ("group", G.PREC_FP32, gsize)):
            ctx.set_bh_walk(g)
            ctx.set_state(p)
            ctx.compute_forces(G.ALGO_BH, prec, eps, 0.5)
            e0 = ctx.diagnostics(eps).total_energy
            ctx.kdk_steps(G.ALGO_BH, prec, eps, 0.5, 1e-3, 500)
            e1 = ctx.diagnostics(eps).total_energy
            drift[name] = abs(e1 - e0) / abs(e0)
    finally:
        ctx.set_bh_walk(-1)
    print(f"group {gsize}: |dE/E| f64 walk {drift['f64']:.2e}, group walk {drift['group']:.2e}")
    assert drift["group"] < 1e-3
    assert drift["group"] <= 2.0 * drift["f64"] + 1e-6


def test_bh_kdk_energy(ctx):
    """Plummer N=2000 with BH theta=0.5: 500 steps at dt=1e-3 keep |dE/E| small (tests/barnes_hut.rs)."""
    p = G.PlummerSphere(2000, seed=42).generate()
    eps = 0.05
    ctx.set_state(p)
    ctx.compute_forces(G.ALGO_BH, G.PREC_FP64, eps, 0.5)
    e0 = ctx.diagnostics(eps).total_energy
    ctx.kdk_steps(G.ALGO_BH, G.PREC_FP64, eps, 0.5, 1e-3, 500)
    e1 = ctx.diagnostics(eps).total_energy
    assert abs(e1 - e0) / abs(e0) < 1e-3

"""Pins the CPU oracle against the reference's own published numbers.

Every value compared here was produced by gravis sim-core itself and is
committed in its repository (artifacts/benchmarks/*.csv, copied into
tests/golden/reference_artifacts.json by tests/golden/make_golden.py), or is a
known answer asserted by one of its unit tests.
"""
import math

import numpy as np
import pytest

import oracle as O


def _close10(a, b):
    # The CSVs print 11 significant digits ({:.10e}); half a unit in the last place.
    return abs(a - b) <= 0.51e-10 * max(abs(b), 1e-300) * 10 or a == b


def test_plummer_initial_row_pins_rng_and_sampler(golden):
    """m1_plummer_1k_diag.csv row 0: ChaCha20 seed 42 + sampler + softened U."""
    row = golden["m1_plummer_1k_diag.csv"]["rows"][0]
    eps = O.plummer_suggested_softening(1000)
    p = O.plummer(1000, 42)
    p.clear_accelerations()
    O.bf_serial(p, eps)
    d = O.diagnostics(p, eps)
    assert f"{d['kinetic_energy']:.10e}" == "1.4655028083e-01"
    for got, want in ((d["kinetic_energy"], row[2]), (d["potential_energy"], row[3]),
                      (d["total_energy"], row[4]), (d["angular_momentum_mag"], row[6])):
        assert _close10(got, want), (got, want)
    assert abs(d["virial_ratio"] - row[8]) <= 5e-7


def test_plummer_1000_steps_pins_bf_and_kdk(golden):
    """All ten 100-step rows of m1_plummer_1k_diag.csv (dt 0.01, BruteForce, KDK)."""
    rows = golden["m1_plummer_1k_diag.csv"]["rows"]
    eps = O.plummer_suggested_softening(1000)
    dt = O.plummer_suggested_dt()
    p = O.plummer(1000, 42)
    p.clear_accelerations()
    O.bf_serial(p, eps)
    g = O.gravity(O.GRAV_BF_GATHER, eps)
    for k in range(1, 11):
        O.kdk_steps(p, g, dt, 100)
        d = O.diagnostics(p, eps)
        want = rows[k]
        assert int(want[0]) == 100 * k
        for got, w in ((d["kinetic_energy"], want[2]), (d["potential_energy"], want[3]),
                       (d["total_energy"], want[4])):
            assert _close10(got, w), (k, got, w)


def test_kepler_rows(golden):
    """m1_kepler_diag.csv: TwoBody e=0.5, dt=T/1e4, 1e5 steps, 10-digit rows."""
    rows = golden["m1_kepler_diag.csv"]["rows"]
    e, a = 0.5, 1.0
    p = O.two_body(0.5, e, a)
    eps = a * (1 - e) * 0.001
    dt = O.lib().orc_two_body_period(a) / 10000.0
    g = O.gravity(O.GRAV_BF, eps)
    p.clear_accelerations()
    O.bf_serial(p, eps)
    d0 = O.diagnostics(p, eps)
    assert _close10(d0["total_energy"], rows[0][4])
    for k in range(1, 11):
        O.kdk_steps(p, g, dt, 10000)
        d = O.diagnostics(p, eps)
        for got, w in ((d["kinetic_energy"], rows[k][2]), (d["potential_energy"], rows[k][3]),
                       (d["total_energy"], rows[k][4]), (d["angular_momentum_mag"], rows[k][6])):
            assert _close10(got, w), (k, got, w)


def test_bh_accuracy_table(golden):
    """m3_accuracy.csv: BH vs BF relative error (N=1000, seed 42, eps 0.05), 7 digits."""
    p0 = O.plummer(1000, 42)
    bf = p0.copy()
    bf.clear_accelerations()
    O.bf_serial(bf, 0.05)
    a = bf.acc()
    for row in golden["m3_accuracy.csv"]["rows"]:
        theta = row[0]
        q = p0.copy()
        q.clear_accelerations()
        O.bh(q, 0.05, theta)
        m2 = (a * a).sum(1)
        e2 = ((q.acc() - a) ** 2).sum(1)
        ok = m2 >= 1e-30
        rel = e2[ok] / m2[ok]
        rms = math.sqrt(rel.sum() / 1000)
        mx = math.sqrt(rel.max())
        assert f"{rms:.6e}" == f"{row[2]:.6e}", (theta, rms, row[2])
        assert f"{mx:.6e}" == f"{row[3]:.6e}", (theta, mx, row[3])


def test_gather_equals_serial_bitwise():
    """The OpenMP gather form is bit-identical to the serial j>i form (gravity.rs:55-78)."""
    p = O.plummer(777, 5)
    q = p.copy()
    p.clear_accelerations()
    q.clear_accelerations()
    O.bf_serial(p, 0.01)
    O.bf_gather(q, 0.01)
    assert np.array_equal(p.acc(), q.acc())


# ---- known answers from the reference's unit tests -------------------------------
def test_force_quarter():
    """gravity.rs:107-120: unit masses at r=2, eps=0 -> a = 0.25."""
    p = O.Particles(2)
    p.x[1] = 2.0
    p.mass[:] = 1.0
    O.bf_serial(p, 0.0)
    assert abs(p.ax[0] - 0.25) < 1e-14
    assert abs(p.ax[0] + p.ax[1]) < 1e-14


def test_octant_indexing():
    """octree.rs:401-413."""
    c = (0.0, 0.0, 0.0)
    assert O.octant(c, -0.5, -0.5, -0.5) == 0
    assert O.octant(c, 0.5, -0.5, -0.5) == 1
    assert O.octant(c, -0.5, 0.5, -0.5) == 2
    assert O.octant(c, 0.5, 0.5, -0.5) == 3
    assert O.octant(c, -0.5, -0.5, 0.5) == 4
    assert O.octant(c, 0.5, 0.5, 0.5) == 7


def test_bh_theta_zero_equals_bf():
    """barnes_hut.rs:219-265: theta = 0 reduces to BruteForce within 1e-12."""
    pts = [(0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 2.0), (0.0, 1.0, 0.0, 1.5), (-1.0, -1.0, 0.5, 0.5),
           (0.5, 0.5, -0.5, 3.0)]
    p = O.Particles(5)
    for i, (x, y, z, m) in enumerate(pts):
        p.x[i], p.y[i], p.z[i], p.mass[i] = x, y, z, m
    q = p.copy()
    O.bh(p, 0.05, 0.0)
    O.bf_serial(q, 0.05)
    assert np.max(np.abs(p.acc() - q.acc())) < 1e-12


def test_sph_kernel_known_answers():
    """sph/kernel.rs tests: support, normalisation, dW/dh vs finite difference."""
    L = O.lib()
    assert L.orc_sph_w(2.0, 1.0) == 0.0
    assert L.orc_sph_w(0.0, 1.0) > 0.0
    # Integral of W over the ball of radius 2h is 1 (kernel.rs:144-160).
    h = 1.0
    r = np.linspace(0.0, 2.0 * h, 20001)
    w = np.array([L.orc_sph_w(x, h) for x in r])
    integral = np.trapezoid(4 * np.pi * r * r * w, r)
    assert abs(integral - 1.0) < 1e-3
    # dW/dh vs central difference (kernel.rs:191-204).
    for rr in (0.3, 0.9, 1.5):
        fd = (L.orc_sph_w(rr, 1.0 + 1e-6) - L.orc_sph_w(rr, 1.0 - 1e-6)) / 2e-6
        assert abs(L.orc_sph_dw_dh(rr, 1.0) - fd) < 1e-5


def test_sph_neighbors_match_brute_force():
    """sph/neighbors.rs:127-178: tree neighbours equal the brute-force set on a 5^3 lattice."""
    n_side, spacing, h = 5, 0.5, 0.8
    n = n_side ** 3
    p = O.Particles(n)
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                p.x[k], p.y[k], p.z[k] = ix * spacing, iy * spacing, iz * spacing
                p.mass[k], p.u[k], p.h[k], p.alpha[k] = 1.0, 1.0, h, 1.0
                p.ptype[k] = O.GAS
                k += 1
    s = O.Sph()
    s.neighbors_only(p, 1.0)
    pos = np.stack([p.x, p.y, p.z], 1)
    for i in range(n):
        d2 = ((pos - pos[i]) ** 2).sum(1)
        bf = np.nonzero(d2 <= (2 * h) ** 2)[0]
        assert np.array_equal(np.sort(s.neighbors(i)), bf)


def test_sph_uniform_density():
    """sph/density.rs:181-251: 8^3 lattice, rho -> m/s^3 = 8 within 5% in the interior."""
    n_side, spacing = 8, 0.5
    n = n_side ** 3
    p = O.Particles(n)
    k = 0
    for ix in range(n_side):
        for iy in range(n_side):
            for iz in range(n_side):
                p.x[k], p.y[k], p.z[k] = ix * spacing, iy * spacing, iz * spacing
                p.mass[k], p.u[k], p.h[k], p.alpha[k] = 1.0, 1.0, 1.0, 1.0
                p.ptype[k] = O.GAS
                k += 1
    s = O.Sph()
    s.compute(p)
    edge = (n_side - 1) * spacing
    errs = []
    for i in range(n):
        m = 2 * p.h[i]
        if min(p.x[i], p.y[i], p.z[i]) < m or max(p.x[i], p.y[i], p.z[i]) > edge - m:
            continue
        errs.append(abs(p.density[i] - 8.0) / 8.0)
    if errs:
        assert np.mean(errs) < 0.05


def test_rng_known_words():
    """ChaCha20 block 0 under an all-zero key is the published keystream 76 b8 e0 ad ...;
    seed_from_u64 feeds PCG32 words as the key, so only the chain is checked here:
    two generators with the same seed agree and different seeds differ."""
    a, b, c = O.Rng(42), O.Rng(42), O.Rng(43)
    xs = [a.next_u64() for _ in range(40)]
    assert xs == [b.next_u64() for _ in range(40)]
    assert xs != [c.next_u64() for _ in range(40)]
    v = O.Rng(7)
    for _ in range(1000):
        x = v.range(0.001, 1.0)
        assert 0.001 <= x < 1.0
